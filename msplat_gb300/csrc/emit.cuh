// Writing a block's tile intersections with coalesced stores.
//
// Each of a block's kEmitThreads threads holds one Gaussian's run: the
// tiles of a rectangle [x0, x0 + w) x [y0, ...) in row-major order, n
// entries, each written as (tile key, Gaussian id).  The runs of a block
// are consecutive in the output (their order is the threads' order, which
// is depth order), so the block's entries form one contiguous range.  The
// threads scan the run lengths into shared memory and then walk that range
// together, entry e + thread for e = 0, kEmitThreads, ...: each finds the
// run holding its entry by binary search over the scanned offsets and
// writes one key and one value, so every store instruction of a warp covers
// 32 consecutive slots, whatever the runs' lengths.  (Spreading one run
// at a time over a warp's lanes, the common alternative, leaves most lanes
// idle when runs are a few tiles long, as most are.)
#pragma once

#include "block_scan.cuh"

namespace msplat {

constexpr int kEmitThreads = 256;

struct EmitShared {
    int64_t off[kEmitThreads + 1];  // exclusive prefix of the run lengths; off[kEmitThreads] = block total
    int g[kEmitThreads];            // Gaussian id written as the value
    uint32_t xy[kEmitThreads];      // x0 | y0 << 16 (tile units)
    int w[kEmitThreads];            // run width in tiles; < 0: a run of key 0 ("no tile")
    int64_t scratch[33];
};

// Emits the block's runs into tkeys / tvals starting at `base` (the first
// slot of the block's range); key = y * gx + x + 1 for tile (x, y), or 0
// for a run with zero_key.  Slots at or past `cap` are not written.  Every
// thread of the block (blockDim.x == kEmitThreads) must call it.
__device__ __forceinline__ void emit_block_runs(EmitShared &sm, int64_t base, int n, int g, int x0, int y0, int w,
                                                bool zero_key, int gx, uint32_t *__restrict__ tkeys,
                                                uint32_t *__restrict__ tvals, int64_t cap) {
    const int t = threadIdx.x;
    int64_t total;
    const int64_t ex = block_exclusive_scan<int64_t>((int64_t)n, sm.scratch, &total);
    sm.off[t] = ex;
    if (t == 0) sm.off[kEmitThreads] = total;
    sm.g[t] = g;
    sm.xy[t] = ((uint32_t)x0 & 0xffffu) | ((uint32_t)y0 << 16);
    sm.w[t] = zero_key ? -max(w, 1) : w;
    __syncthreads();
    const int64_t lim = min(total, cap - base);  // entries of the block that fit (may be <= 0)
    for (int64_t e = t; e < lim; e += kEmitThreads) {
        // the last run starting at or before e (it holds e: the next starts after it)
        int r = 0;
#pragma unroll
        for (int step = kEmitThreads / 2; step > 0; step >>= 1)
            if (sm.off[r + step] <= e) r += step;
        const int k = (int)(e - sm.off[r]);
        const int rw = sm.w[r];
        uint32_t key = 0u;
        if (rw > 0) {
            int ry = (int)(((float)k + 0.5f) / (float)rw);  // k / rw, corrected below
            ry -= (ry * rw > k);
            ry += ((ry + 1) * rw <= k);
            const uint32_t xy = sm.xy[r];
            key = (uint32_t)(((int)(xy >> 16) + ry) * gx + (int)(xy & 0xffffu) + (k - ry * rw) + 1);
        }
        tkeys[base + e] = key;
        tvals[base + e] = (uint32_t)sm.g[r];
    }
}

}  // namespace msplat
