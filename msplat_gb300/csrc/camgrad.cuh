// Deterministic reduction of per-point camera gradients (4 intrinsics +
// 12 extrinsics) used by the projection and EWA backward passes.
//
// The reference adds every point's contribution with float atomics onto the
// same 16 addresses (msplat/src/project_point.cu:107-144,
// msplat/src/ewa_project.cu:206-246): heavily contended and
// order-nondeterministic.  Here each block reduces its points with warp
// shuffles, writes one partial row to scratch, and one block sums the rows
// in a fixed order in double.
#pragma once

#include "common.cuh"

namespace msplat {

constexpr int kCamGradBlocks = 1024;  // upper bound on blocks (scratch rows)
constexpr int kCamGradVals = 16;      // [fx, fy, cx, cy, extr[0..11]]

// Sums vals[] over the block; the block's row goes to partials[blockIdx.x].
// Must be called by every thread of a block of <= 256 threads.
__device__ __forceinline__ void block_partial_16(float (&vals)[kCamGradVals],
                                                 float *__restrict__ partials) {
    __shared__ float red[8][kCamGradVals];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kCamGradVals; ++k) vals[k] = warp_sum(vals[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < kCamGradVals; ++k) red[warp][k] = vals[k];
    }
    __syncthreads();
    if (threadIdx.x < kCamGradVals) {
        float s = 0.0f;
        const int nw = blockDim.x >> 5;
        for (int w = 0; w < nw; ++w) s += red[w][threadIdx.x];
        partials[blockIdx.x * kCamGradVals + threadIdx.x] = s;
    }
}

// Reduce-scatter of the 16 camera-gradient values over a warp: afterwards
// lane l holds the warp total of value l >> 1 (lanes 2i and 2i + 1 the
// same), after 8 + 4 + 2 + 1 + 1 shuffles instead of 16 x 5.
__device__ __forceinline__ float warp_reduce_scatter_16(float (&v)[kCamGradVals]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16, n = 16; o >= 2; o >>= 1, n >>= 1) {
        const bool up = (lane & o) != 0;
        const int h = n >> 1;
#pragma unroll
        for (int k = 0; k < h; ++k) {
            const float send = up ? v[k] : v[k + h];
            const float keep = up ? v[k + h] : v[k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

// Fixed-order sum of `nblocks` partial rows; writes (does not accumulate)
// dL_dintr[4] and dL_dextr[12], either of which may be null.  Thread t sums
// column t % 16 over rows t / 16, t / 16 + 32, ... in double with four
// independent accumulators (so the row loads overlap); the 32 group sums
// of a column are then added in group order.  Deterministic.
constexpr int kCamGradGroups = 32;
constexpr int kCamGradFinalizeThreads = kCamGradGroups * kCamGradVals;

// Launched with one block per camera: block b reads rows
// [b * nblocks, (b + 1) * nblocks) and writes at out_stride * b.
static __global__ void __launch_bounds__(kCamGradFinalizeThreads)
cam_grad_finalize_kernel(int nblocks, const float *__restrict__ partials,
                         float *__restrict__ dL_dintr, float *__restrict__ dL_dextr, int out_stride) {
    __shared__ double part[kCamGradGroups][kCamGradVals];
    partials += (size_t)blockIdx.x * nblocks * kCamGradVals;
    if (dL_dintr) dL_dintr += (size_t)blockIdx.x * out_stride;
    if (dL_dextr) dL_dextr += (size_t)blockIdx.x * out_stride;
    const int k = threadIdx.x % kCamGradVals, grp = threadIdx.x / kCamGradVals;
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    int b = grp;
    for (; b + 3 * kCamGradGroups < nblocks; b += 4 * kCamGradGroups) {
#pragma unroll
        for (int u = 0; u < 4; ++u) s[u] += (double)partials[(b + u * kCamGradGroups) * kCamGradVals + k];
    }
    for (; b < nblocks; b += kCamGradGroups) s[0] += (double)partials[b * kCamGradVals + k];
    part[grp][k] = (s[0] + s[1]) + (s[2] + s[3]);
    __syncthreads();
    if (threadIdx.x >= kCamGradVals) return;
    double t = 0.0;
    for (int g = 0; g < kCamGradGroups; ++g) t += part[g][threadIdx.x];
    if (threadIdx.x < 4) {
        if (dL_dintr) dL_dintr[threadIdx.x] = (float)t;
    } else if (dL_dextr) {
        dL_dextr[threadIdx.x - 4] = (float)t;
    }
}

inline size_t cam_grad_workspace_bytes() {
    return (size_t)kCamGradBlocks * kCamGradVals * sizeof(float);
}

}  // namespace msplat
