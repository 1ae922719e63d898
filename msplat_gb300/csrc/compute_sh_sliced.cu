// SH forward and backward for rows longer than a block's shared memory
// holds (many channels at a high degree); the dispatch in compute_sh.cu
// sends a call here when 32 whole rows do not fit in about 200 KB.
#include "sh_basis.cuh"
#include "sh_dispatch.cuh"

namespace msplat {

// ---- rows longer than a block's shared memory ---------------------------------
// With many channels (C * D floats per Gaussian beyond what 32 Gaussians
// fit in about 200 KB: 16 channels at degree 10, say) the block stages its
// rows a slice of CC channels at a time (sub-rows of CC * D floats, odd
// stride) and runs sh_fwd_kernel's / sh_bwd_kernel's per-channel
// arithmetic on each slice in channel order.  CC is a multiple of the
// channel block, so every value and the direction gradient's sum come out
// of the same operations in the same order as with whole rows.

// Copies floats [0, L) of n rows of `src_stride` floats into shared rows
// of `stride` floats, and back.
__device__ __forceinline__ void stage_slice(float *dst, const float *__restrict__ src, int n, int L, int src_stride,
                                            int stride) {
    for (int e = threadIdx.x; e < n * L; e += blockDim.x) {
        const int p = e / L, k = e - p * L;
        dst[p * stride + k] = __ldcs(src + (size_t)p * src_stride + k);
    }
}

__device__ __forceinline__ void unstage_slice(float *__restrict__ dst, const float *src, int n, int L, int dst_stride,
                                              int stride) {
    for (int e = threadIdx.x; e < n * L; e += blockDim.x) {
        const int p = e / L, k = e - p * L;
        __stcs(dst + (size_t)p * dst_stride + k, src[p * stride + k]);
    }
}

template <int DEG, bool CAM>
__global__ void sh_fwd_sliced_kernel(int P, int C, int CC, const float *__restrict__ shs, ShDirs in,
                                     float *__restrict__ value) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    extern __shared__ float smem[];
    const int CD = C * D;
    const int p0 = blockIdx.x * blockDim.x;
    const int n = min((int)blockDim.x, P - p0);
    const int t = threadIdx.x;
    const int p = p0 + t;
    float cc[3] = {0.f, 0.f, 0.f}, d[3] = {0.f, 0.f, 0.f}, len = 1.f;
    if (CAM) camera_centre(in.extr, cc);
    const bool vis = t < n && sh_direction<CAM>(in, p, cc, d, len);
    for (int s0 = 0; s0 < C; s0 += CC) {
        const int ns = min(CC, C - s0), L = ns * D, stride = L | 1;
        stage_slice(smem, shs + (size_t)p0 * CD + (size_t)s0 * D, n, L, CD, stride);
        __syncthreads();
        if (t < n) {
            float *out = value + (size_t)p * C + s0;
            const float *row = smem + t * stride;
            if (!vis) {
                for (int c = 0; c < ns; ++c) out[c] = 0.f;
            } else {
                for (int c0 = 0; c0 < ns; c0 += kShChanBlock) {
                    float acc[kShChanBlock] = {0.f, 0.f, 0.f, 0.f};
                    const int nc = min(kShChanBlock, ns - c0);
                    sh_basis<DEG, false>(d[0], d[1], d[2], [&](int i, float Y) {
#pragma unroll
                        for (int cb = 0; cb < kShChanBlock; ++cb)
                            if (cb < nc) acc[cb] += Y * row[(c0 + cb) * D + i];
                    });
                    for (int cb = 0; cb < nc; ++cb) out[c0 + cb] = acc[cb];
                }
            }
        }
        __syncthreads();  // the next slice is staged over this one
    }
}

template <int DEG, bool CAM>
__global__ void sh_bwd_sliced_kernel(int P, int C, int CC, const float *__restrict__ shs, ShDirs in,
                                     const float *__restrict__ dL_dval, float *__restrict__ dL_dshs,
                                     float *__restrict__ dL_ddirs) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    extern __shared__ float smem[];
    const int CD = C * D;
    const int p0 = blockIdx.x * blockDim.x;
    const int n = min((int)blockDim.x, P - p0);
    const int t = threadIdx.x;
    const int p = p0 + t;
    float cc[3] = {0.f, 0.f, 0.f}, d[3] = {0.f, 0.f, 0.f}, len = 1.f;
    if (CAM) camera_centre(in.extr, cc);
    const bool vis = t < n && sh_direction<CAM>(in, p, cc, d, len);
    float gdx = 0.f, gdy = 0.f, gdz = 0.f;
    for (int s0 = 0; s0 < C; s0 += CC) {
        const int ns = min(CC, C - s0), L = ns * D, stride = L | 1;
        stage_slice(smem, shs + (size_t)p0 * CD + (size_t)s0 * D, n, L, CD, stride);
        __syncthreads();
        if (t < n) {
            float *row = smem + t * stride;
            if (!vis) {
                for (int k = 0; k < L; ++k) row[k] = 0.f;
            } else {
                for (int c0 = 0; c0 < ns; c0 += kShChanBlock) {
                    float g[kShChanBlock] = {0.f, 0.f, 0.f, 0.f};
                    const int nc = min(kShChanBlock, ns - c0);
                    for (int cb = 0; cb < nc; ++cb) g[cb] = dL_dval[(size_t)p * C + s0 + c0 + cb];
                    sh_basis<DEG, true>(d[0], d[1], d[2], [&](int i, float Y, float yx, float yy, float yz) {
#pragma unroll
                        for (int cb = 0; cb < kShChanBlock; ++cb) {
                            if (cb < nc) {
                                float *slot = row + (c0 + cb) * D + i;
                                const float w = g[cb] * *slot;  // dL/dval * coefficient
                                gdx += w * yx;
                                gdy += w * yy;
                                gdz += w * yz;
                                *slot = g[cb] * Y;  // dL/dsh, written in place
                            }
                        }
                    });
                }
            }
        }
        __syncthreads();
        unstage_slice(dL_dshs + (size_t)p0 * CD + (size_t)s0 * D, smem, n, L, CD, stride);
        __syncthreads();  // the next slice is staged over this one
    }
    if (t < n) {
        if (!CAM) {
            dL_ddirs[3 * p + 0] = gdx;
            dL_ddirs[3 * p + 1] = gdy;
            dL_ddirs[3 * p + 2] = gdz;
        } else {
            float gv[3] = {0.f, 0.f, 0.f};
            if (vis) {
                const float dg = d[0] * gdx + d[1] * gdy + d[2] * gdz;
                gv[0] = (gdx - d[0] * dg) / len;
                gv[1] = (gdy - d[1] * dg) / len;
                gv[2] = (gdz - d[2] * dg) / len;
            }
            in.dxyz[3 * p + 0] = gv[0];
            in.dxyz[3 * p + 1] = gv[1];
            in.dxyz[3 * p + 2] = gv[2];
        }
    }
}

template <int DEG>
void sh_go_sliced(bool backward, int CC, size_t smem, int P, int C, const float *shs, const ShDirs &in,
                  const float *dval, float *out, float *ddirs, cudaStream_t stream) {
    const int blocks = ceil_div(P, kShSlicedPoints);
#define MSPLAT_SH_SLICED(CAM)                                                                                     \
    if (!backward) {                                                                                              \
        cudaFuncSetAttribute(sh_fwd_sliced_kernel<DEG, CAM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        launch(sh_fwd_sliced_kernel<DEG, CAM>, blocks, kShSlicedPoints, smem, stream, P, C, CC, shs, in, out);     \
    } else {                                                                                                      \
        cudaFuncSetAttribute(sh_bwd_sliced_kernel<DEG, CAM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        launch(sh_bwd_sliced_kernel<DEG, CAM>, blocks, kShSlicedPoints, smem, stream, P, C, CC, shs, in, dval, out, \
               ddirs);                                                                                            \
    }
    if (in.xyz) {
        MSPLAT_SH_SLICED(true)
    } else {
        MSPLAT_SH_SLICED(false)
    }
#undef MSPLAT_SH_SLICED
}

#define MSPLAT_SH_SLICED_INST(L)                                                                               \
    template void sh_go_sliced<L>(bool, int, size_t, int, int, const float *, const ShDirs &, const float *, \
                                  float *, float *, cudaStream_t);
MSPLAT_SH_SLICED_INST(0) MSPLAT_SH_SLICED_INST(1) MSPLAT_SH_SLICED_INST(2) MSPLAT_SH_SLICED_INST(3)
MSPLAT_SH_SLICED_INST(4) MSPLAT_SH_SLICED_INST(5) MSPLAT_SH_SLICED_INST(6) MSPLAT_SH_SLICED_INST(7)
MSPLAT_SH_SLICED_INST(8) MSPLAT_SH_SLICED_INST(9) MSPLAT_SH_SLICED_INST(10)
#undef MSPLAT_SH_SLICED_INST

}  // namespace msplat
