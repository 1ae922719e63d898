// Block-wide scans built from warp shuffles (no library dependency).
#pragma once

#include "common.cuh"

namespace msplat {

template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

// Exclusive scan over a block of up to 1024 threads (blockDim.x multiple of
// 32).  `scratch` holds at least 33 elements of T.  Returns the exclusive
// prefix; *total receives the block sum.  Contains __syncthreads().
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *scratch, T *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const T inc = warp_inclusive_scan(v);
    if (lane == 31) scratch[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? scratch[lane] : T(0);
        const T wi = warp_inclusive_scan(w);
        scratch[lane] = wi - w;
        if (lane == 31) scratch[32] = wi;
    }
    __syncthreads();
    const T res = scratch[warp] + inc - v;
    if (total) *total = scratch[32];
    __syncthreads();
    return res;
}

}  // namespace msplat
