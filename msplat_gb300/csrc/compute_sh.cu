// Real spherical harmonics of degree 0..10, forward and backward.
//
// Replaces msplat/src/compute_sh.cu (forward :1600-1637, backward
// :1639-1694), which spells out all 121 basis polynomials and their
// derivatives by hand.  Here the basis is generated by recurrences:
//
//   Y(l,0)  = K(l,0) Q(l,0)
//   Y(l,+m) = K(l,m) Q(l,m) Re((x + i y)^m)      index l^2 + l + m
//   Y(l,-m) = K(l,m) Q(l,m) Im((x + i y)^m)      index l^2 + l - m
//
// with K(l,m) = (-1)^m sqrt((2 - [m == 0]) (2l+1)/(4 pi) (l-m)!/(l+m)!)
// (Condon-Shortley phase) and Q(l,m) the z-part of the associated Legendre
// function from the three-term recurrence
//   Q(m,m) = (2m-1)!!,  Q(m+1,m) = (2m+1) z Q(m,m),
//   Q(l,m) = ((2l-1) z Q(l-1,m) - (l+m-1) s Q(l-2,m)) / (l-m).
// The reference's polynomials are these functions on all of R^3 (not just
// on the sphere) when s = x^2 + y^2 + z^2 for bands l <= 3 and s = 1 for
// bands l >= 4; both are generated so that the direction gradient -- which
// sees the off-sphere shape -- matches the reference as well.
//
// Coefficients are staged per block into shared memory; the backward
// overwrites each row in place with dL/dsh and streams it out.  When a row
// holds an odd number of floats (C * D odd: an even degree and an odd
// channel count, e.g. degree 10 with 3 colours) thread t's word t*CD + k
// falls in a different bank for each of 32 threads without padding, so the
// block's chunk of contiguous rows arrives as ONE bulk copy
// (cp.async.bulk, completing on an mbarrier) and the backward's gradient
// rows leave as one: the whole chunk (24-36 KB) is in flight at once.
// Otherwise the rows are padded to an odd stride and moved by a coalesced
// thread loop; rows longer than 32 of them fit in about 200 KB go to the
// channel-sliced kernels of compute_sh_sliced.cu.
#include <algorithm>

#include "sh_basis.cuh"
#include "sh_dispatch.cuh"

namespace msplat {

// ---- bulk staging ----------------------------------------------------------
// The wait for a bulk copy is bounded like every other device-side wait:
// after `limit` polls (each suspends for at most kShWaitHintNs) the thread
// sets g_sh_wait_error, which the host reads through msplat_wait_error, and
// the block waits once more, for at most kShDrainPolls polls whatever the
// limit, for its copy before it leaves without computing.
static __device__ int g_sh_wait_error;
constexpr uint32_t kShWaitHintNs = 1000;
constexpr int kShDrainPolls = 1 << 21;  // about 2 s at most

int wait_limit_polls();  // process-wide poll limit (msplat_set_wait_limit)

#ifndef MSPLAT_SH_BULK
#define MSPLAT_SH_BULK 1  // bulk copies for odd row lengths (0: the thread loop for all)
#endif
// Bytes of rows per block on the bulk path, forward and backward (degree
// 10, C = 3: 24 and 16 Gaussians, 6 and 9 one-warp blocks per SM).
#ifndef MSPLAT_SH_BULK_KB_FWD
#define MSPLAT_SH_BULK_KB_FWD 36
#endif
#ifndef MSPLAT_SH_BULK_KB_BWD
#define MSPLAT_SH_BULK_KB_BWD 24
#endif
// Kernels with the channel count fixed at 3 (colour) for degrees >= 4.
#ifndef MSPLAT_SH_FIXED_C3
#define MSPLAT_SH_FIXED_C3 1
#endif

__device__ __forceinline__ uint32_t sh_smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool sh_bulk_wait(uint32_t bar, int limit) {
    for (int it = 0; it < limit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0, %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(kShWaitHintNs)
            : "memory");
        if (ok) return true;
    }
    atomicExch(&g_sh_wait_error, 1);
    return false;
}

// The mbarrier of a bulk-staged chunk sits after the rows of `cap` floats.
__device__ __forceinline__ uint64_t *sh_bulk_bar(float *rows, int cap) {
    return reinterpret_cast<uint64_t *>(rows + ((cap + 1) & ~1));
}

// Copies `total` contiguous floats from global (16-byte aligned) into
// shared memory: the largest multiple of 4 by one bulk copy that thread 0
// starts, the rest by plain loads.  Returns (the same in every thread)
// whether the data arrived; the caller leaves without computing if not.
__device__ __forceinline__ bool stage_rows_bulk(float *dst, const float *__restrict__ src, int total, int cap,
                                                int limit) {
    const uint32_t bar = sh_smem_u32(sh_bulk_bar(dst, cap));
    const int nv = total & ~3;
    if (threadIdx.x == 0 && nv > 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(bar),
                     "r"(nv * 4)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         sh_smem_u32(dst)),
                     "l"(src), "r"(nv * 4), "r"(bar)
                     : "memory");
    }
    for (int e = nv + threadIdx.x; e < total; e += blockDim.x) dst[e] = __ldcs(src + e);
    __syncthreads();  // the barrier is initialised before any thread polls it
    const bool ok = nv == 0 || sh_bulk_wait(bar, limit);
    if (__syncthreads_and(ok)) return true;
    if (!ok) sh_bulk_wait(bar, kShDrainPolls);  // the copy may still be writing this block's shared memory
    return false;
}

// Writes `total` floats of shared memory back to global (16-byte aligned):
// one bulk copy from thread 0 for the largest multiple of 4, plain stores
// for the rest.  Every thread of the block calls it after its last write.
__device__ __forceinline__ void unstage_rows_bulk(float *__restrict__ dst, const float *src, int total) {
    const int nv = total & ~3;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // this thread's writes, seen by the copy
    __syncthreads();
    if (threadIdx.x == 0 && nv > 0) {
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(sh_smem_u32(src)),
                     "r"(nv * 4)
                     : "memory");
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // shared memory stays until it is read
    }
    for (int e = nv + threadIdx.x; e < total; e += blockDim.x) __stcs(dst + e, src[e]);
}

// FC > 0: the channel count, fixed at compile time (C is then FC).
template <int DEG, bool CAM, bool BULK, int FC>
__global__ void sh_fwd_kernel(int P, int C_, const float *__restrict__ shs, ShDirs in,
                              float *__restrict__ value, int wait_limit) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    const int C = FC > 0 ? FC : C_;
    extern __shared__ __align__(16) float smem[];
    const int CD = C * D, stride = BULK ? CD : (CD | 1);
    const int p0 = blockIdx.x * blockDim.x;
    const int n = min((int)blockDim.x, P - p0);
    const int t = threadIdx.x;
    const int p = p0 + t;
    // The view direction is read before the rows arrive, so that its
    // latency overlaps the staging.
    float cc[3] = {0.f, 0.f, 0.f}, d[3] = {0.f, 0.f, 0.f}, len = 1.f;
    if (CAM) camera_centre(in.extr, cc);
    const bool vis = t < n && sh_direction<CAM>(in, p, cc, d, len);
    if (BULK) {
        if (!stage_rows_bulk(smem, shs + (size_t)p0 * CD, n * CD, (int)blockDim.x * CD, wait_limit)) return;
    } else {
        stage_rows(smem, shs + (size_t)p0 * CD, n, CD, stride);
        __syncthreads();
    }
    if (t >= n) return;
    const float *row = smem + t * stride;
    float *out = value + (size_t)p * C;
    if (!vis) {
        for (int c = 0; c < C; ++c) out[c] = 0.f;
        return;
    }
    for (int c0 = 0; c0 < C; c0 += kShChanBlock) {
        float acc[kShChanBlock] = {0.f, 0.f, 0.f, 0.f};
        const int nc = min(kShChanBlock, C - c0);
        sh_basis<DEG, false>(d[0], d[1], d[2], [&](int i, float Y) {
#pragma unroll
            for (int cb = 0; cb < kShChanBlock; ++cb)
                if (cb < nc) acc[cb] += Y * row[(c0 + cb) * D + i];
        });
        for (int cb = 0; cb < nc; ++cb) out[c0 + cb] = acc[cb];
    }
}

template <int DEG, bool CAM, bool BULK, int FC>
__global__ void sh_bwd_kernel(int P, int C_, const float *__restrict__ shs, ShDirs in,
                              const float *__restrict__ dL_dval, float *__restrict__ dL_dshs,
                              float *__restrict__ dL_ddirs, int wait_limit) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    const int C = FC > 0 ? FC : C_;
    extern __shared__ __align__(16) float smem[];
    const int CD = C * D, stride = BULK ? CD : (CD | 1);
    const int p0 = blockIdx.x * blockDim.x;
    const int n = min((int)blockDim.x, P - p0);
    const int t = threadIdx.x;
    const int p = p0 + t;
    // The view direction and the first channels' dL/dval are read before
    // the rows arrive, so that their latency overlaps the staging.
    float cc[3] = {0.f, 0.f, 0.f}, d[3] = {0.f, 0.f, 0.f}, len = 1.f;
    if (CAM) camera_centre(in.extr, cc);
    const bool vis = t < n && sh_direction<CAM>(in, p, cc, d, len);
    float g0[kShChanBlock] = {0.f, 0.f, 0.f, 0.f};
    if (vis) {
#pragma unroll
        for (int cb = 0; cb < kShChanBlock; ++cb)
            if (cb < C) g0[cb] = dL_dval[(size_t)p * C + cb];
    }
    if (BULK) {
        if (!stage_rows_bulk(smem, shs + (size_t)p0 * CD, n * CD, (int)blockDim.x * CD, wait_limit)) return;
    } else {
        stage_rows(smem, shs + (size_t)p0 * CD, n, CD, stride);
        __syncthreads();
    }
    if (t < n) {
        float *row = smem + t * stride;
        float gdx = 0.f, gdy = 0.f, gdz = 0.f;
        if (!vis) {
            for (int k = 0; k < CD; ++k) row[k] = 0.f;
        } else {
            for (int c0 = 0; c0 < C; c0 += kShChanBlock) {
                float g[kShChanBlock] = {g0[0], g0[1], g0[2], g0[3]};
                const int nc = min(kShChanBlock, C - c0);
                if (c0 > 0) {
#pragma unroll
                    for (int cb = 0; cb < kShChanBlock; ++cb)
                        g[cb] = cb < nc ? dL_dval[(size_t)p * C + c0 + cb] : 0.f;
                }
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
        if (!CAM) {
            dL_ddirs[3 * p + 0] = gdx;
            dL_ddirs[3 * p + 1] = gdy;
            dL_ddirs[3 * p + 2] = gdz;
        } else {
            // d = v / |v| with v = x - c: dL/dv = (g - d (d . g)) / |v|,
            // which is dL/dx; the camera centre's share (dL/dc = -dL/dv) is
            // folded into the extrinsics by the fused geometry backward.
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
    if (BULK) {
        unstage_rows_bulk(dL_dshs + (size_t)p0 * CD, smem, n * CD);
    } else {
        __syncthreads();
        unstage_rows(dL_dshs + (size_t)p0 * CD, smem, n, CD, stride);
    }
}

// Points per block on the bulk path: the most (at most 256) whose rows fit
// in `kb` KB, rounded down to a multiple of 4 so that every chunk but the
// last starts 16-byte aligned; at least 4.
inline int sh_bulk_block_points(int CD, int kb) {
    const size_t fit = (size_t)kb * 1024 / ((size_t)CD * sizeof(float));
    return (int)std::max<size_t>(4, std::min<size_t>(256, fit) & ~(size_t)3);
}

template <int DEG, bool BULK, int FC>
void sh_go(bool backward, int blocks, int nt, size_t smem, int P, int C, const float *shs, const ShDirs &in,
           const float *dval, float *out, float *ddirs, cudaStream_t stream) {
    const int limit = wait_limit_polls();
#define MSPLAT_SH_GO(CAM)                                                                                           \
    if (!backward) {                                                                                                \
        cudaFuncSetAttribute(sh_fwd_kernel<DEG, CAM, BULK, FC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        launch(sh_fwd_kernel<DEG, CAM, BULK, FC>, blocks, nt, smem, stream, P, C, shs, in, out, limit);                 \
    } else {                                                                                                        \
        cudaFuncSetAttribute(sh_bwd_kernel<DEG, CAM, BULK, FC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        launch(sh_bwd_kernel<DEG, CAM, BULK, FC>, blocks, nt, smem, stream, P, C, shs, in, dval, out, ddirs, limit);    \
    }
    if (in.xyz) {
        MSPLAT_SH_GO(true)
    } else {
        MSPLAT_SH_GO(false)
    }
#undef MSPLAT_SH_GO
}

// Three channels (colour) at degree >= 4 take kernels with the count fixed
// at compile time: the bulk ones at even degrees (C * D odd), the
// thread-loop ones at odd degrees.
template <int DEG, bool BULK>
void sh_go_c(bool backward, int blocks, int nt, size_t smem, int P, int C, const float *shs, const ShDirs &in,
             const float *dval, float *out, float *ddirs, cudaStream_t stream) {
    constexpr bool odd_d = (((DEG + 1) * (DEG + 1)) & 1) != 0;
    if constexpr (DEG >= 4 && MSPLAT_SH_FIXED_C3 && BULK == odd_d) {
        if (C == 3) {
            sh_go<DEG, BULK, 3>(backward, blocks, nt, smem, P, C, shs, in, dval, out, ddirs, stream);
            return;
        }
    }
    sh_go<DEG, BULK, 0>(backward, blocks, nt, smem, P, C, shs, in, dval, out, ddirs, stream);
}

template <int DEG>
int sh_launch(bool backward, int P, int C, const float *shs, const ShDirs &in, const float *dval, float *out,
              float *ddirs, cudaStream_t stream) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    const int CD = C * D;
    if constexpr ((D & 1) != 0 && MSPLAT_SH_BULK) {
        const bool aligned = ((uintptr_t)shs & 15) == 0 && (!backward || ((uintptr_t)out & 15) == 0);
        if ((C & 1) && aligned) {
            const int nt = sh_bulk_block_points(CD, backward ? MSPLAT_SH_BULK_KB_BWD : MSPLAT_SH_BULK_KB_FWD);
            const size_t smem = (size_t)((nt * CD + 1) & ~1) * sizeof(float) + sizeof(uint64_t);
            if (smem <= 200 * 1024) {
                sh_go_c<DEG, true>(backward, ceil_div(P, nt), nt, smem, P, C, shs, in, dval, out, ddirs, stream);
                return check_launch(backward ? "compute_sh_backward" : "compute_sh_forward");
            }
        }
    }
    const int nt = sh_block_points(CD);
    const size_t smem = (size_t)nt * (CD | 1) * sizeof(float);
    if (smem > 200 * 1024) {  // rows longer than a block holds: slices of CC channels
        const size_t per_ch = (size_t)kShSlicedPoints * D * sizeof(float);
        const int CC = std::max<int>(kShChanBlock, (int)((96 * 1024) / per_ch) & ~(kShChanBlock - 1));
        const size_t sm = (size_t)kShSlicedPoints * ((CC * D) | 1) * sizeof(float);
        sh_go_sliced<DEG>(backward, CC, sm, P, C, shs, in, dval, out, ddirs, stream);
        return check_launch(backward ? "compute_sh_backward" : "compute_sh_forward");
    }
    sh_go_c<DEG, false>(backward, ceil_div(P, nt), nt, smem, P, C, shs, in, dval, out, ddirs, stream);
    return check_launch(backward ? "compute_sh_backward" : "compute_sh_forward");
}

cudaError_t sh_wait_error(int reset, int *value, cudaStream_t stream) {
    int h = 0;
    cudaError_t e = cudaMemcpyFromSymbolAsync(&h, g_sh_wait_error, sizeof(int), 0, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e == cudaSuccess && reset && h) {
        const int zero = 0;
        e = cudaMemcpyToSymbolAsync(g_sh_wait_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    }
    if (value) *value = h;
    return e;
}

int sh_dispatch(bool backward, int P, int C, int D, const float *shs, const ShDirs &in, const float *dval,
                float *out, float *ddirs, cudaStream_t stream) {
    int deg = -1;
    for (int l = 0; l <= kMaxShDeg; ++l)
        if ((l + 1) * (l + 1) == D) deg = l;
    if (deg < 0)
        return set_error(MSPLAT_ERR_UNSUPPORTED,
                         "compute_sh: D = %d is not (deg+1)^2 for a degree in 0..10", D);
    switch (deg) {
#define MSPLAT_SH_CASE(L) \
    case L: return sh_launch<L>(backward, P, C, shs, in, dval, out, ddirs, stream);
        MSPLAT_SH_CASE(0) MSPLAT_SH_CASE(1) MSPLAT_SH_CASE(2) MSPLAT_SH_CASE(3)
        MSPLAT_SH_CASE(4) MSPLAT_SH_CASE(5) MSPLAT_SH_CASE(6) MSPLAT_SH_CASE(7)
        MSPLAT_SH_CASE(8) MSPLAT_SH_CASE(9) MSPLAT_SH_CASE(10)
#undef MSPLAT_SH_CASE
    }
    return MSPLAT_ERR_UNSUPPORTED;
}

}  // namespace msplat

using namespace msplat;

extern "C" int msplat_compute_sh_forward(int P, int C, int D, const float *shs,
                                         const float *dirs, const uint8_t *visible,
                                         float *value, msplat_stream_t stream) {
    if (P < 0 || C < 0 || D <= 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_sh_forward: bad sizes P=%d C=%d D=%d", P, C, D);
    if (P == 0 || C == 0) return MSPLAT_OK;
    if (!shs || !dirs || !value)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_sh_forward: null pointer");
    const ShDirs in{dirs, visible, nullptr, nullptr, nullptr, nullptr};
    return sh_dispatch(false, P, C, D, shs, in, nullptr, value, nullptr, stream);
}

extern "C" int msplat_compute_sh_backward(int P, int C, int D, const float *shs,
                                          const float *dirs, const uint8_t *visible,
                                          const float *dL_dvalue, float *dL_dshs,
                                          float *dL_ddirs, msplat_stream_t stream) {
    if (P < 0 || C < 0 || D <= 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_sh_backward: bad sizes P=%d C=%d D=%d", P, C, D);
    if (P == 0) return MSPLAT_OK;
    if (C == 0) return cudaMemsetAsync(dL_ddirs, 0, (size_t)P * 3 * sizeof(float), stream) == cudaSuccess
                           ? MSPLAT_OK : set_error(MSPLAT_ERR_LAUNCH, "compute_sh_backward: memset failed");
    if (!shs || !dirs || !dL_dvalue || !dL_dshs || !dL_ddirs)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_sh_backward: null pointer");
    const ShDirs in{dirs, visible, nullptr, nullptr, nullptr, nullptr};
    return sh_dispatch(true, P, C, D, shs, in, dL_dvalue, dL_dshs, dL_ddirs, stream);
}
