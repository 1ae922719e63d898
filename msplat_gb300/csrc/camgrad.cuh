// Deterministic reduction of per-point camera gradients (4 intrinsics +
// 12 extrinsics) used by the projection and EWA backward passes.
//
// The reference adds every point's contribution with float atomics onto the
// same 16 addresses (msplat/src/project_point.cu:107-144,
// msplat/src/ewa_project.cu:206-246): heavily contended and
// order-nondeterministic.  Here each block reduces its points with warp
// shuffles, writes one partial row to scratch, and a single-warp kernel sums
// the rows in a fixed order in double.
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

// Fixed-order sum of `nblocks` partial rows; writes (does not accumulate)
// dL_dintr[4] and dL_dextr[12], either of which may be null.  Launched with
// 16 warps: warp k sums column k, each lane a strided subset in double, then
// a fixed shuffle tree -- deterministic and latency-parallel.
static __global__ void __launch_bounds__(32 * kCamGradVals)
cam_grad_finalize_kernel(int nblocks, const float *__restrict__ partials,
                         float *__restrict__ dL_dintr, float *__restrict__ dL_dextr) {
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double s = 0.0;
    for (int b = lane; b < nblocks; b += 32) s += (double)partials[b * kCamGradVals + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane != 0) return;
    if (k < 4) {
        if (dL_dintr) dL_dintr[k] = (float)s;
    } else if (dL_dextr) {
        dL_dextr[k - 4] = (float)s;
    }
}

inline size_t cam_grad_workspace_bytes() {
    return (size_t)kCamGradBlocks * kCamGradVals * sizeof(float);
}

}  // namespace msplat
