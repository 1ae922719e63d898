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
#include "sh_dispatch.cuh"

namespace msplat {

constexpr int kMaxShDeg = 10;

// ---- compile-time normalisation table ------------------------------------
constexpr double cx_sqrt(double v) {
    if (v <= 0.0) return 0.0;
    double x = v > 1.0 ? v : 1.0;
    for (int it = 0; it < 64; ++it) x = 0.5 * (x + v / x);
    return x;
}

struct ShNorm {
    float k[kMaxShDeg + 1][kMaxShDeg + 1];
};

constexpr ShNorm make_sh_norm() {
    ShNorm t{};
    const double four_pi = 12.566370614359172953850573533118;
    for (int l = 0; l <= kMaxShDeg; ++l) {
        for (int m = 0; m <= l; ++m) {
            double ratio = 1.0;  // (l-m)! / (l+m)!
            for (int q = l - m + 1; q <= l + m; ++q) ratio /= (double)q;
            double v = (2.0 * l + 1.0) / four_pi * ratio * (m == 0 ? 1.0 : 2.0);
            double k = cx_sqrt(v);
            if (m & 1) k = -k;
            t.k[l][m] = (float)k;
        }
    }
    return t;
}

__constant__ ShNorm kShNorm = make_sh_norm();

constexpr float dfact_odd(int m) {  // (2m-1)!!
    float r = 1.0f;
    for (int q = 2 * m - 1; q > 1; q -= 2) r *= (float)q;
    return r;
}

// ---- basis generation ------------------------------------------------------
// Calls emit(i, Y) for every basis function (forward), or
// emit(i, Y, gx, gy, gz) with the gradient of Y w.r.t. (x, y, z) (backward).
template <int DEG, bool GRAD, typename Emit>
__device__ __forceinline__ void sh_basis(float x, float y, float z, Emit &&emit) {
    const float s_h = x * x + y * y + z * z;  // r^2 for the homogeneous bands
    float cm = 1.0f, sm = 0.0f;               // Re/Im (x + iy)^m
    float cm1 = 0.0f, sm1 = 0.0f;             // ... of m - 1
#pragma unroll
    for (int m = 0; m <= DEG; ++m) {
        if (m > 0) {
            cm1 = cm; sm1 = sm;
            const float c2 = x * cm1 - y * sm1;
            const float s2 = x * sm1 + y * cm1;
            cm = c2; sm = s2;
        }
        // Gradients of the sectoral parts.
        const float dcx = (float)m * cm1, dcy = -(float)m * sm1;
        const float dsx = (float)m * sm1, dsy = (float)m * cm1;
        // Two recurrences: h (s = r^2, used for l <= 3), u (s = 1, l >= 4).
        float qh2 = 0.f, qh1 = 0.f, zh2 = 0.f, zh1 = 0.f, sh2 = 0.f, sh1 = 0.f;
        float qu2 = 0.f, qu1 = 0.f, zu2 = 0.f, zu1 = 0.f;
#pragma unroll
        for (int l = m; l <= DEG; ++l) {
            float qh = 0.f, zh = 0.f, shs = 0.f, qu, zu;
            if (l == m) {
                qu = dfact_odd(m); zu = 0.f;
            } else if (l == m + 1) {
                qu = (float)(2 * m + 1) * z * qu1;
                zu = (float)(2 * m + 1) * qu1;
            } else {
                const float a = (float)(2 * l - 1), b = (float)(l + m - 1), ic = 1.0f / (float)(l - m);
                qu = (a * z * qu1 - b * qu2) * ic;
                zu = (a * (qu1 + z * zu1) - b * zu2) * ic;
            }
            if (l <= 3) {
                if (l == m) {
                    qh = dfact_odd(m); zh = 0.f; shs = 0.f;
                } else if (l == m + 1) {
                    qh = (float)(2 * m + 1) * z * qh1;
                    zh = (float)(2 * m + 1) * qh1;
                    shs = (float)(2 * m + 1) * z * sh1;
                } else {
                    const float a = (float)(2 * l - 1), b = (float)(l + m - 1), ic = 1.0f / (float)(l - m);
                    qh = (a * z * qh1 - b * s_h * qh2) * ic;
                    zh = (a * (qh1 + z * zh1) - b * s_h * zh2) * ic;
                    shs = (a * z * sh1 - b * (qh2 + s_h * sh2)) * ic;
                }
            }
            // Pick the band's form.
            const float q = (l <= 3) ? qh : qu;
            const float qz = (l <= 3) ? zh : zu;
            const float qs = (l <= 3) ? shs : 0.f;
            const float k = kShNorm.k[l][m];
            if (m == 0) {
                const int i = l * l + l;
                if constexpr (GRAD) {
                    emit(i, k * q, k * (2.f * x * qs), k * (2.f * y * qs), k * (qz + 2.f * z * qs));
                } else {
                    emit(i, k * q);
                }
            } else {
                const int ic_ = l * l + l + m, is_ = l * l + l - m;
                const float kq = k * q;
                if constexpr (GRAD) {
                    // grad Q = (2x qs, 2y qs, qz + 2z qs)
                    const float gqx = k * 2.f * x * qs, gqy = k * 2.f * y * qs, gqz = k * (qz + 2.f * z * qs);
                    emit(ic_, kq * cm, cm * gqx + kq * dcx, cm * gqy + kq * dcy, cm * gqz);
                    emit(is_, kq * sm, sm * gqx + kq * dsx, sm * gqy + kq * dsy, sm * gqz);
                } else {
                    emit(ic_, kq * cm);
                    emit(is_, kq * sm);
                }
            }
            qu2 = qu1; qu1 = qu; zu2 = zu1; zu1 = zu;
            qh2 = qh1; qh1 = qh; zh2 = zh1; zh1 = zh; sh2 = sh1; sh1 = shs;
        }
    }
}

constexpr int kShChanBlock = 4;

// Copies n contiguous rows of CD floats from global memory into shared
// memory rows of `stride` floats (odd, against bank conflicts).  The chunk is
// read as a flat, coalesced stream -- 16-byte vectors when aligned -- with
// many loads in flight per thread.
__device__ __forceinline__ void stage_rows(float *dst, const float *__restrict__ src, int n, int CD,
                                           int stride) {
    const int total = n * CD;
    int done = 0;
    if ((((uintptr_t)src) & 15) == 0) {
        const int nv = total >> 2;
        const float4 *s4 = reinterpret_cast<const float4 *>(src);
#pragma unroll 4
        for (int v = threadIdx.x; v < nv; v += blockDim.x) {
            const float4 q = __ldcs(s4 + v);
            int e = v << 2;
            int p = e / CD, k = e - p * CD;
            const float vals[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                dst[p * stride + k] = vals[u];
                if (++k == CD) { k = 0; ++p; }
            }
        }
        done = nv << 2;
    }
    for (int e = done + threadIdx.x; e < total; e += blockDim.x) {
        const int p = e / CD;
        dst[p * stride + (e - p * CD)] = __ldcs(src + e);
    }
}

__device__ __forceinline__ void unstage_rows(float *__restrict__ dst, const float *src, int n, int CD,
                                             int stride) {
    const int total = n * CD;
    int done = 0;
    if ((((uintptr_t)dst) & 15) == 0) {
        const int nv = total >> 2;
        float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll 4
        for (int v = threadIdx.x; v < nv; v += blockDim.x) {
            int e = v << 2;
            int p = e / CD, k = e - p * CD;
            float vals[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                vals[u] = src[p * stride + k];
                if (++k == CD) { k = 0; ++p; }
            }
            __stcs(d4 + v, make_float4(vals[0], vals[1], vals[2], vals[3]));
        }
        done = nv << 2;
    }
    for (int e = done + threadIdx.x; e < total; e += blockDim.x) {
        const int p = e / CD;
        __stcs(dst + e, src[p * stride + (e - p * CD)]);
    }
}

__device__ __forceinline__ void camera_centre(const float *__restrict__ e, float (&c)[3]) {
#pragma unroll
    for (int j = 0; j < 3; ++j) c[j] = -(__ldg(e + j) * __ldg(e + 3) + __ldg(e + 4 + j) * __ldg(e + 7) +
                                         __ldg(e + 8 + j) * __ldg(e + 11));
}

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

// Points per block so that a block's staged rows stay under ~96 KB.
inline int sh_block_points(int CD) {
    const int stride = CD | 1;
    int nt = 256;
    while (nt > 32 && (size_t)nt * stride * sizeof(float) > 96 * 1024) nt >>= 1;
    return nt;
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
