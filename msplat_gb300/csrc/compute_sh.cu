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
// Coefficients are staged per block into shared memory with coalesced
// loads (rows padded to an odd stride against bank conflicts); the
// backward overwrites each row in place with dL/dsh and streams it out.
#include "sh_basis.cuh"
#include "sh_dispatch.cuh"

namespace msplat {

// Direction of point p and whether it is visible; n = |x - c| in camera mode.
template <bool CAM>
__device__ __forceinline__ bool sh_direction(const ShDirs &in, int p, const float (&cc)[3], float (&d)[3],
                                             float &n) {
    if (CAM) {
        if (in.depth[p] == 0.0f) return false;
        const float dx = in.xyz[3 * p] - cc[0], dy = in.xyz[3 * p + 1] - cc[1], dz = in.xyz[3 * p + 2] - cc[2];
        n = sqrtf(dx * dx + dy * dy + dz * dz);
        d[0] = dx / n;
        d[1] = dy / n;
        d[2] = dz / n;
        return true;
    }
    if (in.visible && !in.visible[p]) return false;
    d[0] = in.dirs[3 * p];
    d[1] = in.dirs[3 * p + 1];
    d[2] = in.dirs[3 * p + 2];
    n = 1.0f;
    return true;
}

template <int DEG, bool CAM>
__global__ void sh_fwd_kernel(int P, int C, const float *__restrict__ shs, ShDirs in,
                              float *__restrict__ value) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    extern __shared__ float smem[];
    const int CD = C * D, stride = CD | 1;
    const int p0 = blockIdx.x * blockDim.x;
    const int n = min((int)blockDim.x, P - p0);
    stage_rows(smem, shs + (size_t)p0 * CD, n, CD, stride);
    __syncthreads();
    const int t = threadIdx.x;
    if (t >= n) return;
    const int p = p0 + t;
    const float *row = smem + t * stride;
    float *out = value + (size_t)p * C;
    float cc[3] = {0.f, 0.f, 0.f}, d[3], len;
    if (CAM) camera_centre(in.extr, cc);
    if (!sh_direction<CAM>(in, p, cc, d, len)) {
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

template <int DEG, bool CAM>
__global__ void sh_bwd_kernel(int P, int C, const float *__restrict__ shs, ShDirs in,
                              const float *__restrict__ dL_dval, float *__restrict__ dL_dshs,
                              float *__restrict__ dL_ddirs) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    extern __shared__ float smem[];
    const int CD = C * D, stride = CD | 1;
    const int p0 = blockIdx.x * blockDim.x;
    const int n = min((int)blockDim.x, P - p0);
    stage_rows(smem, shs + (size_t)p0 * CD, n, CD, stride);
    __syncthreads();
    const int t = threadIdx.x;
    if (t < n) {
        const int p = p0 + t;
        float *row = smem + t * stride;
        float gdx = 0.f, gdy = 0.f, gdz = 0.f;
        float cc[3] = {0.f, 0.f, 0.f}, d[3], len = 1.f;
        if (CAM) camera_centre(in.extr, cc);
        const bool vis = sh_direction<CAM>(in, p, cc, d, len);
        if (!vis) {
            for (int k = 0; k < CD; ++k) row[k] = 0.f;
        } else {
            for (int c0 = 0; c0 < C; c0 += kShChanBlock) {
                float g[kShChanBlock] = {0.f, 0.f, 0.f, 0.f};
                const int nc = min(kShChanBlock, C - c0);
                for (int cb = 0; cb < nc; ++cb) g[cb] = dL_dval[(size_t)p * C + c0 + cb];
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
    __syncthreads();
    unstage_rows(dL_dshs + (size_t)p0 * CD, smem, n, CD, stride);
}

template <int DEG>
int sh_launch(bool backward, int P, int C, const float *shs, const ShDirs &in, const float *dval, float *out,
              float *ddirs, cudaStream_t stream) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    const int CD = C * D;
    const int nt = sh_block_points(CD);
    const size_t smem = (size_t)nt * (CD | 1) * sizeof(float);
    if (smem > 200 * 1024)
        return set_error(MSPLAT_ERR_UNSUPPORTED, "compute_sh: C*D = %d too large", CD);
    const int blocks = ceil_div(P, nt);
#define MSPLAT_SH_GO(CAM)                                                                                     \
    if (!backward) {                                                                                          \
        cudaFuncSetAttribute(sh_fwd_kernel<DEG, CAM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        launch(sh_fwd_kernel<DEG, CAM>, blocks, nt, smem, stream, P, C, shs, in, out);                        \
    } else {                                                                                                  \
        cudaFuncSetAttribute(sh_bwd_kernel<DEG, CAM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        launch(sh_bwd_kernel<DEG, CAM>, blocks, nt, smem, stream, P, C, shs, in, dval, out, ddirs);           \
    }
    if (in.xyz) {
        MSPLAT_SH_GO(true)
    } else {
        MSPLAT_SH_GO(false)
    }
#undef MSPLAT_SH_GO
    return check_launch(backward ? "compute_sh_backward" : "compute_sh_forward");
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
