// Writing a block's tile intersections with coalesced stores.
//
// Each of a block's kEmitThreads threads holds one Gaussian's run: the
// tiles of a rectangle [x0, x0 + w) x [y0, ...) in row-major order, n
// entries, each written as (tile key, Gaussian id).  The runs of a block
// are consecutive in the output (their order is the threads' order, which
// is depth order), so the block's entries form one contiguous range.  The
// threads scan the run lengths into shared memory and then walk that range
// together in groups of four consecutive slots per thread: each finds the
// run holding its group's first entry by binary search over the scanned
// offsets and writes four keys and four values with 16-byte stores, so
// every store instruction of a warp covers 128 consecutive slots, whatever
// the runs' lengths.  (Spreading one run
// at a time over a warp's lanes, the common alternative, leaves most lanes
// idle when runs are a few tiles long, as most are.)
#pragma once

#include "block_scan.cuh"
#include "cull.cuh"

namespace msplat {

constexpr int kEmitThreads = 256;

struct EmitShared {
    int32_t off[kEmitThreads + 1];  // exclusive prefix of the run lengths (saturated at INT32_MAX)
    int g[kEmitThreads];            // Gaussian id written as the value
    uint32_t xy[kEmitThreads];      // x0 | y0 << 16 (tile units)
    int w[kEmitThreads];            // run width in tiles; < 0: a run of key 0 ("no tile")
    int64_t scratch[33];
};

// Key and value of entry k of run r.
__device__ __forceinline__ void emit_entry(const EmitShared &sm, int r, int k, int gx, uint32_t &key, uint32_t &val) {
    const int rw = sm.w[r];
    key = 0u;
    if (rw > 0) {
        int ry = (int)(((float)k + 0.5f) / (float)rw);  // k / rw, corrected below
        ry -= (ry * rw > k);
        ry += ((ry + 1) * rw <= k);
        const uint32_t xy = sm.xy[r];
        key = (uint32_t)(((int)(xy >> 16) + ry) * gx + (int)(xy & 0xffffu) + (k - ry * rw) + 1);
    }
    val = (uint32_t)sm.g[r];
}

// Emits the block's runs into tkeys / tvals starting at `base` (the first
// slot of the block's range); key = y * gx + x + 1 for tile (x, y), or 0
// for a run with zero_key.  Slots at or past `cap` are not written.  Every
// thread of the block (blockDim.x == kEmitThreads) must call it.
// tkeys / tvals must be 16-byte aligned.  Each thread takes groups of four
// consecutive slots starting on a multiple of four (16-byte stores); the
// run of a group's first entry is found by binary search over the scanned
// offsets, the next three by stepping past the runs that end before them.
// Written slots lie below cap <= INT32_MAX, so offsets saturated there
// still compare correctly with every entry that is written.
__device__ __forceinline__ void emit_block_runs(EmitShared &sm, int64_t base, int n, int g, int x0, int y0, int w,
                                                bool zero_key, int gx, uint32_t *__restrict__ tkeys,
                                                uint32_t *__restrict__ tvals, int64_t cap) {
    const int t = threadIdx.x;
    int64_t total;
    const int64_t ex = block_exclusive_scan<int64_t>((int64_t)n, sm.scratch, &total);
    sm.off[t] = (int32_t)min(ex, (int64_t)INT32_MAX);
    if (t == 0) sm.off[kEmitThreads] = (int32_t)min(total, (int64_t)INT32_MAX);
    sm.g[t] = g;
    sm.xy[t] = ((uint32_t)x0 & 0xffffu) | ((uint32_t)y0 << 16);
    sm.w[t] = zero_key ? -max(w, 1) : w;
    __syncthreads();
    const int lim = (int)max((int64_t)0, min(total, cap - base));  // entries of the block that fit
    // entries before the first slot on a multiple of four, one per thread
    const int head = min(lim, (int)((4 - (base & 3)) & 3));
    if (t < head) {
        int r = 0;
#pragma unroll
        for (int step = kEmitThreads / 2; step > 0; step >>= 1)
            if (sm.off[r + step] <= t) r += step;
        uint32_t key, val;
        emit_entry(sm, r, t - sm.off[r], gx, key, val);
        tkeys[base + t] = key;
        tvals[base + t] = val;
    }
    for (int e0 = head + 4 * t; e0 < lim; e0 += 4 * kEmitThreads) {
        int r = 0;
#pragma unroll
        for (int step = kEmitThreads / 2; step > 0; step >>= 1)
            if (sm.off[r + step] <= e0) r += step;
        uint32_t key[4], val[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int e = e0 + u;
            if (e < lim) {
                while (sm.off[r + 1] <= e) ++r;  // (skips runs of no entries too)
                emit_entry(sm, r, e - sm.off[r], gx, key[u], val[u]);
            }
        }
        if (e0 + 4 <= lim) {
            *reinterpret_cast<uint4 *>(tkeys + base + e0) = make_uint4(key[0], key[1], key[2], key[3]);
            *reinterpret_cast<uint4 *>(tvals + base + e0) = make_uint4(val[0], val[1], val[2], val[3]);
        } else {
            for (int u = 0; u < lim - e0; ++u) {
                tkeys[base + e0 + u] = key[u];
                tvals[base + e0 + u] = val[u];
            }
        }
    }
}

// ------------------------------------------------------------------------
// The same for runs culled row by row (row_span): a run is the tiles its
// reach keeps in each row of its rectangle, row after row.  Two levels:
// the rows of the block's runs are numbered (a scan of the row counts),
// and taken 256 at a time; each thread evaluates one row's span, the
// spans' lengths are scanned, and the chunk's entries are written four
// consecutive slots per thread (binary search over the chunk's row offsets
// for the group's first entry, as emit_block_runs does over runs).
struct EmitRowShared {
    RowReach reach[kEmitThreads];   // per run: centre, conic, threshold
    int x0[kEmitThreads], x1[kEmitThreads], y0[kEmitThreads];
    int g[kEmitThreads];
    int ru[kEmitThreads + 1];       // exclusive prefix of the runs' row counts
    int e[kEmitThreads + 1];        // per row of the chunk: exclusive prefix of the span lengths
    uint32_t kb[kEmitThreads];      // per row of the chunk: key of its first entry
    int rg[kEmitThreads];           // per row of the chunk: its run's Gaussian id
    int iscratch[33];
};

// `allotted` = the slots the count kernel gave the block (its runs' row
// span sums); entries past it, or at or past `cap`, are not written, so a
// disagreement could never write outside the block's range (the span is
// evaluated identically in both kernels, so none arises).
__device__ __forceinline__ void emit_block_rows(EmitRowShared &sm, int64_t base, int64_t allotted, bool valid,
                                                const RowReach &reach, int x0, int y0, int x1, int y1, int g, int gx,
                                                uint32_t *__restrict__ tkeys, uint32_t *__restrict__ tvals,
                                                int64_t cap) {
    const int t = threadIdx.x;
    const int h = valid && x0 < x1 ? max(0, y1 - y0) : 0;  // rows: 256 x 32767 at most, within int
    int rows;
    const int ru = block_exclusive_scan<int>(h, sm.iscratch, &rows);
    sm.ru[t] = ru;
    if (t == 0) sm.ru[kEmitThreads] = rows;
    sm.reach[t] = reach;
    sm.x0[t] = x0;
    sm.x1[t] = x1;
    sm.y0[t] = y0;
    sm.g[t] = g;
    __syncthreads();
    const int64_t lim_all = max((int64_t)0, min(allotted, cap - base));
    int64_t done = 0;  // entries of the earlier chunks (the same in every thread)
    for (int u0 = 0; u0 < rows; u0 += kEmitThreads) {
        const int u = u0 + t;
        int w = 0;
        uint32_t kb = 0u;
        int rg = 0;
        if (u < rows) {
            int r = 0;
#pragma unroll
            for (int step = kEmitThreads / 2; step > 0; step >>= 1)
                if (sm.ru[r + step] <= u) r += step;
            const int ty = sm.y0[r] + (u - sm.ru[r]);
            int xa, xb;
            row_span(sm.reach[r], ty, sm.x0[r], sm.x1[r], xa, xb);
            w = xb - xa;
            kb = (uint32_t)(ty * gx + xa + 1);
            rg = sm.g[r];
        }
        int tot;  // a chunk's entries: 256 rows of at most 32767 tiles, within int
        const int ex = block_exclusive_scan<int>(w, sm.iscratch, &tot);
        sm.e[t] = ex;
        sm.kb[t] = kb;
        sm.rg[t] = rg;
        if (t == 0) sm.e[kEmitThreads] = tot;
        __syncthreads();
        const int64_t cbase = base + done;
        const int lim = (int)max((int64_t)0, min((int64_t)tot, lim_all - done));
        const int head = min(lim, (int)((4 - (cbase & 3)) & 3));
        if (t < head) {
            int q = 0;
#pragma unroll
            for (int step = kEmitThreads / 2; step > 0; step >>= 1)
                if (sm.e[q + step] <= t) q += step;
            tkeys[cbase + t] = sm.kb[q] + (uint32_t)(t - sm.e[q]);
            tvals[cbase + t] = (uint32_t)sm.rg[q];
        }
        for (int e0 = head + 4 * t; e0 < lim; e0 += 4 * kEmitThreads) {
            int q = 0;
#pragma unroll
            for (int step = kEmitThreads / 2; step > 0; step >>= 1)
                if (sm.e[q + step] <= e0) q += step;
            uint32_t key[4], val[4];
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                const int e = e0 + v;
                if (e < lim) {
                    while (sm.e[q + 1] <= e) ++q;  // (skips rows of no entries too)
                    key[v] = sm.kb[q] + (uint32_t)(e - sm.e[q]);
                    val[v] = (uint32_t)sm.rg[q];
                }
            }
            if (e0 + 4 <= lim) {
                *reinterpret_cast<uint4 *>(tkeys + cbase + e0) = make_uint4(key[0], key[1], key[2], key[3]);
                *reinterpret_cast<uint4 *>(tvals + cbase + e0) = make_uint4(val[0], val[1], val[2], val[3]);
            } else {
                for (int v = 0; v < lim - e0; ++v) {
                    tkeys[cbase + e0 + v] = key[v];
                    tvals[cbase + e0 + v] = val[v];
                }
            }
        }
        done += tot;
        __syncthreads();  // the chunk's rows are rewritten by the next chunk
    }
}

}  // namespace msplat
