// Real spherical harmonics of degree 0..10 by recurrences (the basis
// generator shared by the SH kernels of compute_sh.cu and the batched
// preprocess of batch.cu), plus the shared-memory staging of coefficient
// rows.  The derivation is in compute_sh.cu.
#pragma once

#include "common.cuh"

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

// static: every translation unit that includes this header gets its own copy
static __constant__ ShNorm kShNorm = make_sh_norm();

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

// Points per block so that a block's staged rows stay under ~96 KB.
inline int sh_block_points(int CD) {
    const int stride = CD | 1;
    int nt = 256;
    while (nt > 32 && (size_t)nt * stride * sizeof(float) > 96 * 1024) nt >>= 1;
    return nt;
}


}  // namespace msplat
