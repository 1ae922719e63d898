/*
 * oracle.c -- CPU restatement of the reference rasteriser (pointrix-project/
 * msplat) for parity testing.  TEST INFRASTRUCTURE ONLY: imported by tests/,
 * __graft_entry__.smoke() and the cpu_baseline / reference arm of bench.py,
 * never by the product path.
 *
 * Built with -ffp-contract=off so that every fused multiply-add here is an
 * explicit fmaf().  The GPU build (like the reference's, setup.py:39) lets
 * the compiler contract a*b + c into FMAs; the float32 forward stages below
 * reproduce that with helpers whose contraction pattern is a runtime switch
 * (oracle_set_fma_mode) pinned by the GPU parity tests.  Divisions, square
 * roots and exponentials are IEEE here; the GPU uses the fast-math
 * approximations, so integer outputs that depend on them (radius, ncontrib)
 * come with an "ambiguous" flag marking values within rounding reach of a
 * decision boundary.
 *
 * Each function cites the reference code it restates.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define TILE 16

/* ------------------------------------------------------------------ FMA */
/* 0: in a*b + c*d the first product is fused, fma(a, b, c*d)
 * 1: the second product is fused, fma(c, d, a*b)
 * 2: no contraction                                                      */
static int g_mode = 0;

void oracle_set_fma_mode(int m) { g_mode = m; }
int oracle_get_fma_mode(void) { return g_mode; }

/* Host threads for the timed CPU baseline.  1 (the default, used by every
 * parity check) runs each loop serially in index order; n > 1 splits the
 * per-Gaussian loops into n static chunks and the pixel loops into
 * interleaved rows.  Outputs are identical except for the order in which
 * the double-precision camera and per-Gaussian blend gradients are summed. */
static int g_threads = 1;
void oracle_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int oracle_get_threads(void) {
#ifdef _OPENMP
    return g_threads;
#else
    return 1;
#endif
}
#ifdef _OPENMP
#include <omp.h>
#define PARFOR _Pragma("omp parallel for schedule(static) num_threads(g_threads)")
static int thread_id(void) { return omp_get_thread_num(); }
static int team_size(void) { return omp_get_num_threads(); }
#else
#define PARFOR
static int thread_id(void) { return 0; }
static int team_size(void) { return 1; }
#endif

static inline float madd(float a, float b, float c) { return g_mode == 2 ? a * b + c : fmaf(a, b, c); }

static inline float sum2(float a, float b, float c, float d) {
    switch (g_mode) {
        case 0: return fmaf(a, b, c * d);
        case 1: return fmaf(c, d, a * b);
        default: return a * b + c * d;
    }
}

static inline float sum3(float a, float b, float c, float d, float e, float f) {
    return g_mode == 2 ? (a * b + c * d) + e * f : fmaf(e, f, sum2(a, b, c, d));
}

/* a*b - c*d */
static inline float msub(float a, float b, float c, float d) {
    switch (g_mode) {
        case 0: return fmaf(a, b, -(c * d));
        case 1: return fmaf(-c, d, a * b);
        default: return a * b - c * d;
    }
}

/* ------------------------------------------------------- glm-style mat3 */
/* Column-major m[j][i] = column j, row i; product as glm's mat3 operator*. */
typedef struct { float m[3][3]; } mat3f;

static mat3f m3_cols(float a00, float a01, float a02, float a10, float a11, float a12, float a20,
                     float a21, float a22) {
    mat3f r;
    r.m[0][0] = a00; r.m[0][1] = a01; r.m[0][2] = a02;
    r.m[1][0] = a10; r.m[1][1] = a11; r.m[1][2] = a12;
    r.m[2][0] = a20; r.m[2][1] = a21; r.m[2][2] = a22;
    return r;
}

static mat3f m3_mul(mat3f A, mat3f B) {
    mat3f R;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i)
            R.m[j][i] = sum3(A.m[0][i], B.m[j][0], A.m[1][i], B.m[j][1], A.m[2][i], B.m[j][2]);
    return R;
}

static mat3f m3_t(mat3f A) {
    mat3f R;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) R.m[j][i] = A.m[i][j];
    return R;
}

/* ---------------------------------------------------------- projection */
static inline void cam_point(const float *e, float x, float y, float z, float *t) {
    t[0] = sum3(e[0], x, e[1], y, e[2], z) + e[3];
    t[1] = sum3(e[4], x, e[5], y, e[6], z) + e[7];
    t[2] = sum3(e[8], x, e[9], y, e[10], z) + e[11];
}

/* msplat/src/project_point.cu:13-57 */
void oracle_project_point_forward(int P, const float *xyz, const float *intr, const float *extr, int W,
                                  int H, float nearest, float extent, float *uv, float *depth) {
    PARFOR
    for (int i = 0; i < P; ++i) {
        float t[3];
        cam_point(extr, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], t);
        const float inv = (float)(1.0 / ((double)t[2] + 1e-7));
        const float u = (float)((double)madd(intr[0] * t[0], inv, intr[2]) - 0.5);
        const float v = (float)((double)madd(intr[1] * t[1], inv, intr[3]) - 0.5);
        int culled = (nearest > 0) && (t[2] <= nearest);
        if (extent > 0) {
            const float xlo = (float)((double)((1.0f - extent) * (float)W) * 0.5);
            const float xhi = (float)((double)((1.0f + extent) * (float)W) * 0.5);
            const float ylo = (float)((double)((1.0f - extent) * (float)H) * 0.5);
            const float yhi = (float)((double)((1.0f + extent) * (float)H) * 0.5);
            culled |= (u < xlo) || (u > xhi) || (v < ylo) || (v > yhi);
        }
        uv[2 * i] = culled ? 0.f : u;
        uv[2 * i + 1] = culled ? 0.f : v;
        depth[i] = culled ? 0.f : t[2];
    }
}

/* msplat/src/project_point.cu:59-145, in double.  dL_dintr/dL_dextr may be
 * NULL; when given they are written. */
void oracle_project_point_backward(int P, const float *xyz, const float *intr, const float *extr,
                                   const float *depth, const float *dL_duv, const float *dL_ddepth,
                                   double *dL_dxyz, double *dL_dintr, double *dL_dextr) {
    double gi[4] = {0, 0, 0, 0}, ge[12];
    memset(ge, 0, sizeof(ge));
    const double fx = intr[0], fy = intr[1];
    double *part = (double *)calloc((size_t)g_threads * 16, sizeof(double));
#ifdef _OPENMP
#pragma omp parallel num_threads(g_threads)
#endif
    {
        const int tid = thread_id(), nth = team_size();
        const int i0 = (int)((int64_t)P * tid / nth), i1 = (int)((int64_t)P * (tid + 1) / nth);
        double *pi = part + 16 * tid, *pe = pi + 4;
        for (int i = i0; i < i1; ++i) {
            dL_dxyz[3 * i] = dL_dxyz[3 * i + 1] = dL_dxyz[3 * i + 2] = 0.0;
            if (depth[i] == 0.0f) continue;
            const double p[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
            double t[3];
            for (int r = 0; r < 3; ++r)
                t[r] = extr[4 * r] * p[0] + extr[4 * r + 1] * p[1] + extr[4 * r + 2] * p[2] + extr[4 * r + 3];
            const double gu = dL_duv[2 * i], gv = dL_duv[2 * i + 1], gd = dL_ddepth[i];
            const double dt[3] = {fx * gu / t[2], fy * gv / t[2],
                                  -(fx * t[0] * gu + fy * t[1] * gv) / (t[2] * t[2]) + gd};
            for (int c = 0; c < 3; ++c)
                dL_dxyz[3 * i + c] = extr[c] * dt[0] + extr[4 + c] * dt[1] + extr[8 + c] * dt[2];
            pi[0] += t[0] / t[2] * gu;
            pi[1] += t[1] / t[2] * gv;
            pi[2] += gu;
            pi[3] += gv;
            for (int r = 0; r < 3; ++r) {
                for (int c = 0; c < 3; ++c) pe[4 * r + c] += dt[r] * p[c];
                pe[4 * r + 3] += dt[r];
            }
        }
    }
    for (int t = 0; t < g_threads; ++t) {
        for (int k = 0; k < 4; ++k) gi[k] += part[16 * t + k];
        for (int k = 0; k < 12; ++k) ge[k] += part[16 * t + 4 + k];
    }
    free(part);
    if (dL_dintr) memcpy(dL_dintr, gi, sizeof(gi));
    if (dL_dextr) memcpy(dL_dextr, ge, sizeof(ge));
}

/* --------------------------------------------------------------- cov3d */
/* Contraction choices of the covariance code, where products are shared
 * between entries and the compiler's pairing can differ from the global
 * mode: bit 0 flips the pairing of the rotation's sums, bit 1 of its
 * differences, bit 2 of the Sigma = M^T M products.  Pinned by the GPU
 * parity tests. */
static int g_cov_variant = 0;

void oracle_set_cov_variant(int v) { g_cov_variant = v; }

static inline float sum2_v(float a, float b, float c, float d, int flip) {
    if (g_mode == 2) return a * b + c * d;
    return (flip ^ (g_mode == 1)) ? fmaf(c, d, a * b) : fmaf(a, b, c * d);
}

static inline float msub_v(float a, float b, float c, float d, int flip) {
    if (g_mode == 2) return a * b - c * d;
    return (flip ^ (g_mode == 1)) ? fmaf(-c, d, a * b) : fmaf(a, b, -(c * d));
}

/* bit 3: products shared between a sum and a difference (x*y, r*z, ...)
 * are not fused at all; bit 4: the same for the squares. */
static inline float osum(float a, float b, float c, float d, int flip, int nofuse) {
    return nofuse ? a * b + c * d : sum2_v(a, b, c, d, flip);
}

static inline float odif(float a, float b, float c, float d, int flip, int nofuse) {
    return nofuse ? a * b - c * d : msub_v(a, b, c, d, flip);
}

static mat3f quat_rot_cols(float r, float x, float y, float z) {
    const int fs = g_cov_variant & 1, fd = (g_cov_variant >> 1) & 1;
    const int no = (g_cov_variant >> 3) & 1, nq = (g_cov_variant >> 4) & 1;
    return m3_cols(1.f - 2.f * osum(y, y, z, z, fs, nq), 2.f * odif(x, y, r, z, fd, no), 2.f * osum(x, z, r, y, fs, no),
                   2.f * osum(x, y, r, z, fs, no), 1.f - 2.f * osum(x, x, z, z, fs, nq), 2.f * odif(y, z, r, x, fd, no),
                   2.f * odif(x, z, r, y, fd, no), 2.f * osum(y, z, r, x, fs, no), 1.f - 2.f * osum(x, x, y, y, fs, nq));
}

static mat3f m3_mul_v(mat3f A, mat3f B, int flip) {
    mat3f R;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
            const float p = sum2_v(A.m[0][i], B.m[j][0], A.m[1][i], B.m[j][1], flip);
            R.m[j][i] = g_mode == 2 ? p + A.m[2][i] * B.m[j][2] : fmaf(A.m[2][i], B.m[j][2], p);
        }
    return R;
}

/* msplat/src/compute_cov3d.cu:14-58, 119-129 */
void oracle_compute_cov3d_forward(int P, const float *scales, const float *q, const uint8_t *visible,
                                  float *cov3d) {
    PARFOR
    for (int i = 0; i < P; ++i) {
        float *o = cov3d + 6 * i;
        if (visible && !visible[i]) {
            memset(o, 0, 6 * sizeof(float));
            continue;
        }
        const float *s = scales + 3 * i;
        const mat3f S = m3_cols(s[0], 0.f, 0.f, 0.f, s[1], 0.f, 0.f, 0.f, s[2]);
        const mat3f R = quat_rot_cols(q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]);
        const mat3f M = m3_mul(S, R);
        const mat3f Sig = m3_mul_v(m3_t(M), M, (g_cov_variant >> 2) & 1);
        o[0] = Sig.m[0][0]; o[1] = Sig.m[0][1]; o[2] = Sig.m[0][2];
        o[3] = Sig.m[1][1]; o[4] = Sig.m[1][2]; o[5] = Sig.m[2][2];
    }
}

/* msplat/src/compute_cov3d.cu:60-117, 131-147, in double: Sigma = A A^T with
 * A = Rs diag(s), Rs the standard rotation of q = (r, x, y, z). */
void oracle_compute_cov3d_backward(int P, const float *scales, const float *q, const uint8_t *visible,
                                   const float *dL_dcov, double *dL_ds, double *dL_dq) {
    PARFOR
    for (int i = 0; i < P; ++i) {
        double *ds = dL_ds + 3 * i, *dq = dL_dq + 4 * i;
        ds[0] = ds[1] = ds[2] = 0;
        dq[0] = dq[1] = dq[2] = dq[3] = 0;
        if (visible && !visible[i]) continue;
        const double r = q[4 * i], x = q[4 * i + 1], y = q[4 * i + 2], z = q[4 * i + 3];
        const double s[3] = {scales[3 * i], scales[3 * i + 1], scales[3 * i + 2]};
        const double Rs[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)},
                                 {2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)},
                                 {2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)}};
        const float *g = dL_dcov + 6 * i;
        const double G[3][3] = {{g[0], 0.5 * g[1], 0.5 * g[2]},
                                {0.5 * g[1], g[3], 0.5 * g[4]},
                                {0.5 * g[2], 0.5 * g[4], g[5]}};
        double A[3][3], dA[3][3], Gr[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) A[a][b] = Rs[a][b] * s[b];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                dA[a][b] = 2 * (G[a][0] * A[0][b] + G[a][1] * A[1][b] + G[a][2] * A[2][b]);
        for (int b = 0; b < 3; ++b) {
            ds[b] = dA[0][b] * Rs[0][b] + dA[1][b] * Rs[1][b] + dA[2][b] * Rs[2][b];
            for (int a = 0; a < 3; ++a) Gr[a][b] = dA[a][b] * s[b];
        }
        dq[0] = 2 * z * (Gr[1][0] - Gr[0][1]) + 2 * y * (Gr[0][2] - Gr[2][0]) + 2 * x * (Gr[2][1] - Gr[1][2]);
        dq[1] = 2 * y * (Gr[0][1] + Gr[1][0]) + 2 * z * (Gr[0][2] + Gr[2][0]) + 2 * r * (Gr[2][1] - Gr[1][2]) -
                4 * x * (Gr[1][1] + Gr[2][2]);
        dq[2] = 2 * x * (Gr[0][1] + Gr[1][0]) + 2 * r * (Gr[0][2] - Gr[2][0]) + 2 * z * (Gr[1][2] + Gr[2][1]) -
                4 * y * (Gr[0][0] + Gr[2][2]);
        dq[3] = 2 * r * (Gr[1][0] - Gr[0][1]) + 2 * x * (Gr[0][2] + Gr[2][0]) + 2 * y * (Gr[1][2] + Gr[2][1]) -
                4 * z * (Gr[0][0] + Gr[1][1]);
    }
}

/* ----------------------------------------------------------------- EWA */
/* msplat/include/utils.h:17-36 */
static void get_rect(float px, float py, int r, int gx, int gy, int *x0, int *y0, int *x1, int *y1) {
    const float fr = (float)r;
#define CLAMP_I(v, hi) ((v) < 0 ? 0 : ((v) > (hi) ? (hi) : (v)))
    const float a = (px - fr) / 16.0f, b = (py - fr) / 16.0f;
    const float c = ((px + fr) + 16.0f - 1.0f) / 16.0f, d = ((py + fr) + 16.0f - 1.0f) / 16.0f;
    int ia = (a != a) ? 0 : (a > 2e9f ? 2000000000 : (a < -2e9f ? -2000000000 : (int)a));
    int ib = (b != b) ? 0 : (b > 2e9f ? 2000000000 : (b < -2e9f ? -2000000000 : (int)b));
    int ic = (c != c) ? 0 : (c > 2e9f ? 2000000000 : (c < -2e9f ? -2000000000 : (int)c));
    int id = (d != d) ? 0 : (d > 2e9f ? 2000000000 : (d < -2e9f ? -2000000000 : (int)d));
    *x0 = CLAMP_I(ia, gx);
    *y0 = CLAMP_I(ib, gy);
    *x1 = CLAMP_I(ic, gx);
    *y1 = CLAMP_I(id, gy);
#undef CLAMP_I
}

/* msplat/src/ewa_project.cu:16-83.  ambiguous[i] = 1 where the radius (and
 * with it tiles) is within rounding reach of a different integer, given
 * that the GPU divides and takes square roots approximately.
 *
 * Two-branch form: where ambiguous[i] is set, radius_alt[i] / tiles_alt[i]
 * (when given) hold the other outcome a correct implementation can reach --
 * ceil(3 sqrt(lambda)) one integer up or down (the side the value lies
 * nearer to), with its rectangle; radius_alt = 0 means "invisible" (empty
 * rectangle, or det within rounding reach of 0 and the primary visible).
 * Elsewhere radius_alt = -1 (no alternative).  conic_alt [P,3] (when
 * given) holds the conic of a visible alternative (zeros otherwise), which
 * differs from conic[] only where the primary outcome is invisible. */
void oracle_ewa_project_forward_alt(int P, const float *xyz, const float *cov3d, const float *intr,
                                    const float *extr, const float *uv, int W, int H, const uint8_t *visible,
                                    float *conic, int32_t *radius, int32_t *tiles, uint8_t *ambiguous,
                                    int32_t *radius_alt, int32_t *tiles_alt, float *conic_alt) {
    const int gx = (W + TILE - 1) / TILE, gy = (H + TILE - 1) / TILE;
    const float fx = intr[0], fy = intr[1];
    PARFOR
    for (int i = 0; i < P; ++i) {
        conic[3 * i] = conic[3 * i + 1] = conic[3 * i + 2] = 0.f;
        radius[i] = 0;
        tiles[i] = 0;
        if (ambiguous) ambiguous[i] = 0;
        if (radius_alt) radius_alt[i] = -1;
        if (tiles_alt) tiles_alt[i] = -1;
        if (conic_alt) conic_alt[3 * i] = conic_alt[3 * i + 1] = conic_alt[3 * i + 2] = 0.f;
        if (visible && !visible[i]) continue;
        float t[3];
        cam_point(extr, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], t);
        const mat3f J = m3_cols(fx / t[2], 0.f, 0.f, 0.f, fy / t[2], 0.f, -(fx * t[0]) / (t[2] * t[2]),
                                -(fy * t[1]) / (t[2] * t[2]), 0.f);
        const mat3f Wm = m3_cols(extr[0], extr[4], extr[8], extr[1], extr[5], extr[9], extr[2], extr[6], extr[10]);
        const mat3f T = m3_mul(J, Wm);
        const float *v = cov3d + 6 * i;
        const mat3f V = m3_cols(v[0], v[1], v[2], v[1], v[3], v[4], v[2], v[4], v[5]);
        const mat3f c2 = m3_mul(m3_mul(T, V), m3_t(T));
        const float a = c2.m[0][0] + 0.3f, b = c2.m[0][1], c = c2.m[1][1] + 0.3f;
        const float det = msub(a, c, b, b);
        const int det_amb = fabsf(det) <= 1e-5f * (fabsf(a * c) + b * b);
        int amb = det_amb;
        if (det == 0.0f) {
            /* the GPU evaluates det with the same operations: an exact 0
             * there too, so no alternative */
            if (ambiguous) ambiguous[i] = (uint8_t)amb;
            continue;
        }
        const float mid = 0.5f * (a + c);
        const float disc = sqrtf(fmaxf(0.1f, madd(mid, mid, -det)));
        const float l1 = mid + disc, l2 = mid - disc;
        const float vr = 3.f * sqrtf(fmaxf(l1, l2));
        const float r = ceilf(vr);
        const int r_amb = fabsf(vr - rintf(vr)) <= 1e-4f * fmaxf(1.0f, vr);
        if (r_amb) amb = 1;
        int x0, y0, x1, y1;
        get_rect(uv[2 * i], uv[2 * i + 1], (int)r, gx, gy, &x0, &y0, &x1, &y1);
        if (ambiguous) ambiguous[i] = (uint8_t)amb;
        const int n = (x1 - x0) * (y1 - y0);
        if (r_amb && radius_alt) {
            /* vr just above an integer k: ceil gives k + 1, the other k;
             * just below (or at) k: ceil gives k, the other k + 1 */
            const int ra = vr > rintf(vr) ? (int)r - 1 : (int)r + 1;
            int ax0, ay0, ax1, ay1;
            get_rect(uv[2 * i], uv[2 * i + 1], ra, gx, gy, &ax0, &ay0, &ax1, &ay1);
            const int na = (ax1 - ax0) * (ay1 - ay0);
            radius_alt[i] = na == 0 ? 0 : ra;
            if (tiles_alt) tiles_alt[i] = na;
        } else if (det_amb && radius_alt && n != 0) {
            radius_alt[i] = 0;
            if (tiles_alt) tiles_alt[i] = 0;
        }
        const float inv = 1.f / det;
        if (conic_alt && radius_alt && radius_alt[i] > 0) {
            conic_alt[3 * i] = c * inv;
            conic_alt[3 * i + 1] = -b * inv;
            conic_alt[3 * i + 2] = a * inv;
        }
        if (n == 0) continue;
        conic[3 * i] = c * inv;
        conic[3 * i + 1] = -b * inv;
        conic[3 * i + 2] = a * inv;
        radius[i] = (int)r;
        tiles[i] = n;
    }
}

void oracle_ewa_project_forward(int P, const float *xyz, const float *cov3d, const float *intr,
                                const float *extr, const float *uv, int W, int H, const uint8_t *visible,
                                float *conic, int32_t *radius, int32_t *tiles, uint8_t *ambiguous) {
    oracle_ewa_project_forward_alt(P, xyz, cov3d, intr, extr, uv, W, H, visible, conic, radius, tiles, ambiguous,
                                   NULL, NULL, NULL);
}

/* msplat/src/ewa_project.cu:85-252, in double. */
void oracle_ewa_project_backward(int P, const float *xyz, const float *cov3d, const float *intr,
                                 const float *extr, const int32_t *radius, const float *dL_dconic,
                                 double *dL_dxyz, double *dL_dcov3d, double *dL_dintr, double *dL_dextr) {
    double gi[4] = {0, 0, 0, 0}, ge[12];
    memset(ge, 0, sizeof(ge));
    const double fx = intr[0], fy = intr[1];
    double R[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R[r][c] = extr[4 * r + c];
    double *part = (double *)calloc((size_t)g_threads * 16, sizeof(double));
#ifdef _OPENMP
#pragma omp parallel num_threads(g_threads)
#endif
    {
        const int tid = thread_id(), nth = team_size();
        const int i0 = (int)((int64_t)P * tid / nth), i1 = (int)((int64_t)P * (tid + 1) / nth);
        double *pi = part + 16 * tid, *pe = pi + 4;
        for (int i = i0; i < i1; ++i) {
            double *dx = dL_dxyz + 3 * i, *dv = dL_dcov3d + 6 * i;
            memset(dx, 0, 3 * sizeof(double));
            memset(dv, 0, 6 * sizeof(double));
            if (!(radius[i] > 0)) continue;
            const double p[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
            double t[3];
            for (int r = 0; r < 3; ++r) t[r] = R[r][0] * p[0] + R[r][1] * p[1] + R[r][2] * p[2] + extr[4 * r + 3];
            const double J00 = fx / t[2], J11 = fy / t[2];
            const double J02 = -fx * t[0] / (t[2] * t[2]), J12 = -fy * t[1] / (t[2] * t[2]);
            double T0[3], T1[3];
            for (int k = 0; k < 3; ++k) {
                T0[k] = J00 * R[0][k] + J02 * R[2][k];
                T1[k] = J11 * R[1][k] + J12 * R[2][k];
            }
            const float *vf = cov3d + 6 * i;
            const double V[3][3] = {{vf[0], vf[1], vf[2]}, {vf[1], vf[3], vf[4]}, {vf[2], vf[4], vf[5]}};
            double VT0[3], VT1[3];
            for (int k = 0; k < 3; ++k) {
                VT0[k] = V[k][0] * T0[0] + V[k][1] * T0[1] + V[k][2] * T0[2];
                VT1[k] = V[k][0] * T1[0] + V[k][1] * T1[1] + V[k][2] * T1[2];
            }
            const double a = T0[0] * VT0[0] + T0[1] * VT0[1] + T0[2] * VT0[2] + 0.3;
            const double b = T0[0] * VT1[0] + T0[1] * VT1[1] + T0[2] * VT1[2];
            const double c = T1[0] * VT1[0] + T1[1] * VT1[1] + T1[2] * VT1[2] + 0.3;
            const double det = a * c - b * b;
            if (det == 0.0) continue;
            const double g0 = dL_dconic[3 * i], g1 = dL_dconic[3 * i + 1], g2 = dL_dconic[3 * i + 2];
            const double inv2 = 1.0 / (det * det);
            const double da = inv2 * (-c * c * g0 + b * c * g1 + (det - a * c) * g2);
            const double db = inv2 * (2 * b * c * g0 - (det + 2 * b * b) * g1 + 2 * a * b * g2);
            const double dc = inv2 * ((det - a * c) * g0 + a * b * g1 - a * a * g2);
            dv[0] = T0[0] * T0[0] * da + T0[0] * T1[0] * db + T1[0] * T1[0] * dc;
            dv[3] = T0[1] * T0[1] * da + T0[1] * T1[1] * db + T1[1] * T1[1] * dc;
            dv[5] = T0[2] * T0[2] * da + T0[2] * T1[2] * db + T1[2] * T1[2] * dc;
            dv[1] = 2 * T0[0] * T0[1] * da + (T0[0] * T1[1] + T0[1] * T1[0]) * db + 2 * T1[0] * T1[1] * dc;
            dv[2] = 2 * T0[0] * T0[2] * da + (T0[0] * T1[2] + T0[2] * T1[0]) * db + 2 * T1[0] * T1[2] * dc;
            dv[4] = 2 * T0[1] * T0[2] * da + (T0[1] * T1[2] + T0[2] * T1[1]) * db + 2 * T1[1] * T1[2] * dc;
            double dT0[3], dT1[3];
            for (int k = 0; k < 3; ++k) {
                dT0[k] = 2 * VT0[k] * da + VT1[k] * db;
                dT1[k] = VT0[k] * db + 2 * VT1[k] * dc;
            }
            const double dJ00 = R[0][0] * dT0[0] + R[0][1] * dT0[1] + R[0][2] * dT0[2];
            const double dJ02 = R[2][0] * dT0[0] + R[2][1] * dT0[1] + R[2][2] * dT0[2];
            const double dJ11 = R[1][0] * dT1[0] + R[1][1] * dT1[1] + R[1][2] * dT1[2];
            const double dJ12 = R[2][0] * dT1[0] + R[2][1] * dT1[1] + R[2][2] * dT1[2];
            const double iz = 1.0 / t[2], iz2 = iz * iz, iz3 = iz2 * iz;
            const double dt[3] = {-fx * iz2 * dJ02, -fy * iz2 * dJ12,
                                  -fx * iz2 * dJ00 - fy * iz2 * dJ11 + 2 * fx * t[0] * iz3 * dJ02 +
                                      2 * fy * t[1] * iz3 * dJ12};
            for (int k = 0; k < 3; ++k) dx[k] = R[0][k] * dt[0] + R[1][k] * dt[1] + R[2][k] * dt[2];
            pi[0] += iz * dJ00 - t[0] * iz2 * dJ02;
            pi[1] += iz * dJ11 - t[1] * iz2 * dJ12;
            for (int k = 0; k < 3; ++k) {
                pe[k] += J00 * dT0[k] + p[k] * dt[0];
                pe[4 + k] += J11 * dT1[k] + p[k] * dt[1];
                pe[8 + k] += J02 * dT0[k] + J12 * dT1[k] + p[k] * dt[2];
            }
            pe[3] += dt[0];
            pe[7] += dt[1];
            pe[11] += dt[2];
        }
    }
    for (int t = 0; t < g_threads; ++t) {
        for (int k = 0; k < 4; ++k) gi[k] += part[16 * t + k];
        for (int k = 0; k < 12; ++k) ge[k] += part[16 * t + 4 + k];
    }
    free(part);
    if (dL_dintr) memcpy(dL_dintr, gi, sizeof(gi));
    if (dL_dextr) memcpy(dL_dextr, ge, sizeof(ge));
}

/* ------------------------------------------------------------------ SH */
/* Real SH, degrees 0..10, as the functions on R^3 that the reference spells
 * out (msplat/src/compute_sh.cu:116-503 forward, :505-1598 backward):
 * Y(l,0) = K Q, Y(l,+-m) = K Q Re/Im (x + iy)^m with the associated-Legendre
 * z-part Q from the three-term recurrence, s = x^2+y^2+z^2 in the recurrence
 * for l <= 3 and s = 1 for l >= 4; K includes the Condon-Shortley phase. */
static void sh_basis_d(int deg, double x, double y, double z, double *Y, double *Yx, double *Yy, double *Yz) {
    const double sh = x * x + y * y + z * z;
    double cm = 1, sm = 0, cm1 = 0, sm1 = 0;
    for (int m = 0; m <= deg; ++m) {
        if (m > 0) {
            cm1 = cm; sm1 = sm;
            const double c2 = x * cm1 - y * sm1, s2 = x * sm1 + y * cm1;
            cm = c2; sm = s2;
        }
        double qh1 = 0, qh2 = 0, zh1 = 0, zh2 = 0, sh1 = 0, sh2 = 0;
        double qu1 = 0, qu2 = 0, zu1 = 0, zu2 = 0;
        for (int l = m; l <= deg; ++l) {
            double qu, zu, qh = 0, zh = 0, shv = 0;
            if (l == m) {
                double d = 1;
                for (int k = 2 * m - 1; k > 1; k -= 2) d *= k;
                qu = d; zu = 0; qh = d; zh = 0; shv = 0;
            } else if (l == m + 1) {
                qu = (2 * m + 1) * z * qu1; zu = (2 * m + 1) * qu1;
                qh = (2 * m + 1) * z * qh1; zh = (2 * m + 1) * qh1; shv = (2 * m + 1) * z * sh1;
            } else {
                const double a = 2 * l - 1, b = l + m - 1, c = l - m;
                qu = (a * z * qu1 - b * qu2) / c;
                zu = (a * (qu1 + z * zu1) - b * zu2) / c;
                qh = (a * z * qh1 - b * sh * qh2) / c;
                zh = (a * (qh1 + z * zh1) - b * sh * zh2) / c;
                shv = (a * z * sh1 - b * (qh2 + sh * sh2)) / c;
            }
            const int hom = l <= 3;
            const double q = hom ? qh : qu, qz = hom ? zh : zu, qs = hom ? shv : 0;
            double ratio = 1;
            for (int k = l - m + 1; k <= l + m; ++k) ratio /= k;
            double K = sqrt((2.0 * l + 1) / (4.0 * M_PI) * ratio * (m == 0 ? 1.0 : 2.0));
            if (m & 1) K = -K;
            const double gqx = K * 2 * x * qs, gqy = K * 2 * y * qs, gqz = K * (qz + 2 * z * qs);
            if (m == 0) {
                const int i = l * l + l;
                Y[i] = K * q; Yx[i] = gqx; Yy[i] = gqy; Yz[i] = gqz;
            } else {
                const int ic = l * l + l + m, is = l * l + l - m;
                Y[ic] = K * q * cm;
                Yx[ic] = cm * gqx + K * q * m * cm1;
                Yy[ic] = cm * gqy - K * q * m * sm1;
                Yz[ic] = cm * gqz;
                Y[is] = K * q * sm;
                Yx[is] = sm * gqx + K * q * m * sm1;
                Yy[is] = sm * gqy + K * q * m * cm1;
                Yz[is] = sm * gqz;
            }
            qu2 = qu1; qu1 = qu; zu2 = zu1; zu1 = zu;
            qh2 = qh1; qh1 = qh; zh2 = zh1; zh1 = zh; sh2 = sh1; sh1 = shv;
        }
    }
}

/* Basis values (and gradients) for n directions: Y[n][D], G[n][D][3]. */
void oracle_sh_basis(int n, int deg, const double *dirs, double *Y, double *G) {
    const int D = (deg + 1) * (deg + 1);
    double y[121], gx[121], gy[121], gz[121];
    for (int i = 0; i < n; ++i) {
        sh_basis_d(deg, dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2], y, gx, gy, gz);
        for (int k = 0; k < D; ++k) {
            Y[(size_t)i * D + k] = y[k];
            if (G) {
                G[((size_t)i * D + k) * 3 + 0] = gx[k];
                G[((size_t)i * D + k) * 3 + 1] = gy[k];
                G[((size_t)i * D + k) * 3 + 2] = gz[k];
            }
        }
    }
}

static int sh_deg_of(int D) {
    for (int l = 0; l <= 10; ++l)
        if ((l + 1) * (l + 1) == D) return l;
    return -1;
}

/* msplat/src/compute_sh.cu:1600-1637 */
int oracle_compute_sh_forward(int P, int C, int D, const float *shs, const float *dirs, const uint8_t *visible,
                              double *value) {
    const int deg = sh_deg_of(D);
    if (deg < 0) return 1;
    PARFOR
    for (int i = 0; i < P; ++i) {
        double y[121], gx[121], gy[121], gz[121];
        for (int c = 0; c < C; ++c) value[(size_t)i * C + c] = 0;
        if (visible && !visible[i]) continue;
        sh_basis_d(deg, dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2], y, gx, gy, gz);
        for (int c = 0; c < C; ++c) {
            double s = 0;
            const float *row = shs + ((size_t)i * C + c) * D;
            for (int k = 0; k < D; ++k) s += y[k] * row[k];
            value[(size_t)i * C + c] = s;
        }
    }
    return 0;
}

/* msplat/src/compute_sh.cu:1639-1694 */
int oracle_compute_sh_backward(int P, int C, int D, const float *shs, const float *dirs, const uint8_t *visible,
                               const float *dL_dval, double *dL_dshs, double *dL_ddirs) {
    const int deg = sh_deg_of(D);
    if (deg < 0) return 1;
    PARFOR
    for (int i = 0; i < P; ++i) {
        double y[121], gx[121], gy[121], gz[121];
        double *dd = dL_ddirs + 3 * i;
        dd[0] = dd[1] = dd[2] = 0;
        for (int k = 0; k < C * D; ++k) dL_dshs[(size_t)i * C * D + k] = 0;
        if (visible && !visible[i]) continue;
        sh_basis_d(deg, dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2], y, gx, gy, gz);
        for (int c = 0; c < C; ++c) {
            const double g = dL_dval[(size_t)i * C + c];
            const float *row = shs + ((size_t)i * C + c) * D;
            for (int k = 0; k < D; ++k) {
                dL_dshs[((size_t)i * C + c) * D + k] = g * y[k];
                dd[0] += g * row[k] * gx[k];
                dd[1] += g * row[k] * gy[k];
                dd[2] += g * row[k] * gz[k];
            }
        }
    }
    return 0;
}

/* ---------------------------------------------------------------- sort */
typedef struct { int64_t key; int64_t pos; int32_t val; } kv_t;

static int kv_cmp(const void *pa, const void *pb) {
    const kv_t *a = (const kv_t *)pa, *b = (const kv_t *)pb;
    if (a->key != b->key) return a->key < b->key ? -1 : 1;
    return a->pos < b->pos ? -1 : (a->pos > b->pos);
}

/* Number of intersections: tiles_cumsum[P-1] of the int32 inclusive scan
 * (msplat/sort_gaussian.py:42, msplat/src/sort_gaussian.cu:89-91). */
int64_t oracle_num_intersects(int P, const int32_t *tiles) {
    int32_t s = 0;
    for (int i = 0; i < P; ++i) s = (int32_t)((uint32_t)s + (uint32_t)tiles[i]);
    return P > 0 ? (int64_t)s : 0;
}

/* msplat/sort_gaussian.py:8-54 with msplat/src/sort_gaussian.cu:17-71:
 * keys (tile << 32 | sign-extended depth bits) at the scanned offsets of a
 * zero-filled buffer, stable sort (torch.sort on int64), gather, tile
 * boundaries.  Writes keys_sorted if non-NULL.  Returns I. */
int64_t oracle_sort_gaussian(int P, const float *uv, const float *depth, int W, int H, const int32_t *radius,
                             const int32_t *tiles, int32_t *idx_sorted, int32_t *tile_range, int64_t *keys_sorted) {
    const int gx = (W + TILE - 1) / TILE, gy = (H + TILE - 1) / TILE, nt = gx * gy;
    const int64_t I = oracle_num_intersects(P, tiles);
    memset(tile_range, 0, sizeof(int32_t) * 2 * (size_t)nt);
    if (I <= 0) return I < 0 ? 0 : I;
    kv_t *kv = (kv_t *)calloc((size_t)I, sizeof(kv_t));
    PARFOR
    for (int64_t k = 0; k < I; ++k) kv[k].pos = k;
    /* start offsets: exclusive int32 scan of tiles (wrapping like the
     * reference's int32 cumsum) */
    int32_t *start = (int32_t *)malloc(sizeof(int32_t) * (P > 0 ? P : 1));
    int32_t cum = 0;
    for (int g = 0; g < P; ++g) {
        start[g] = cum;
        cum = (int32_t)((uint32_t)cum + (uint32_t)tiles[g]);
    }
    PARFOR
    for (int g = 0; g < P; ++g) {
        if (radius[g] <= 0) continue;
        int x0, y0, x1, y1;
        get_rect(uv[2 * g], uv[2 * g + 1], radius[g], gx, gy, &x0, &y0, &x1, &y1);
        int32_t d;
        memcpy(&d, &depth[g], 4);
        int64_t cur = start[g];
        for (int ty = y0; ty < y1; ++ty)
            for (int tx = x0; tx < x1; ++tx) {
                if (cur >= 0 && cur < I) {
                    kv[cur].key = ((int64_t)(ty * gx + tx) << 32) | (int64_t)d;
                    kv[cur].val = g;
                }
                ++cur;
            }
    }
    free(start);
    /* Sort by (key, position): a stable sort by key.  When every key's high
     * word is a tile index, a stable counting pass by tile followed by a
     * sort of each tile's run gives the same order as one global sort. */
    int64_t bad = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(g_threads) reduction(+ : bad)
#endif
    for (int64_t k = 0; k < I; ++k) {
        const int64_t t = kv[k].key >> 32;
        bad += (t < 0 || t >= nt);
    }
    if (bad == 0) {
        int64_t *off = (int64_t *)calloc((size_t)nt + 1, sizeof(int64_t));
        int64_t *hist = (int64_t *)calloc((size_t)g_threads * nt, sizeof(int64_t));  /* [thread][tile] */
        kv_t *tmp = (kv_t *)malloc((size_t)I * sizeof(kv_t));
#ifdef _OPENMP
#pragma omp parallel num_threads(g_threads)
#endif
        {
            const int tid = thread_id(), nth = team_size();
            const int64_t k0 = I * tid / nth, k1 = I * (tid + 1) / nth;
            int64_t *h = hist + (size_t)tid * nt;
            for (int64_t k = k0; k < k1; ++k) h[kv[k].key >> 32]++;
#ifdef _OPENMP
#pragma omp barrier
#pragma omp single
#endif
            {
                /* exclusive offsets in (tile, thread) order keep the scatter stable */
                int64_t run = 0;
                for (int t = 0; t < nt; ++t) {
                    off[t] = run;
                    for (int q = 0; q < nth; ++q) {
                        const int64_t c = hist[(size_t)q * nt + t];
                        hist[(size_t)q * nt + t] = run;
                        run += c;
                    }
                }
                off[nt] = run;
            }
            for (int64_t k = k0; k < k1; ++k) tmp[h[kv[k].key >> 32]++] = kv[k];
        }
        free(kv);
        kv = tmp;
        free(hist);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(g_threads)
#endif
        for (int t = 0; t < nt; ++t)
            qsort(kv + off[t], (size_t)(off[t + 1] - off[t]), sizeof(kv_t), kv_cmp);
        free(off);
    } else {
        qsort(kv, (size_t)I, sizeof(kv_t), kv_cmp);
    }
    PARFOR
    for (int64_t k = 0; k < I; ++k) {
        idx_sorted[k] = kv[k].val;
        if (keys_sorted) keys_sorted[k] = kv[k].key;
    }
    PARFOR
    for (int64_t k = 0; k < I; ++k) {
        const int t = (int)(kv[k].key >> 32);
        if (t < 0 || t >= nt) continue;
        if (k == 0 || (int)(kv[k - 1].key >> 32) != t) tile_range[2 * t] = (int32_t)k;
        if (k == I - 1 || (int)(kv[k + 1].key >> 32) != t) tile_range[2 * t + 1] = (int32_t)(k + 1);
    }
    free(kv);
    return I;
}

/* --------------------------------------------------------------- blend */
/* power = -0.5 (a dx^2 + c dy^2) - b dx dy with the compiler's contraction. */
static inline float blend_power(float a, float b, float c, float dx, float dy) {
    const float s = sum2(a * dx, dx, c * dy, dy);
    switch (g_mode) {
        case 0: return fmaf(-0.5f, s, -((b * dx) * dy));
        case 1: return fmaf(-(b * dx), dy, -0.5f * s);
        default: return -0.5f * s - (b * dx) * dy;
    }
}

#define NEAR(x, t) (fabsf((x) - (t)) <= 1e-5f * fabsf(t) + 1e-7f)

/* msplat/src/alpha_blending.cu:16-110 (float32, IEEE exp).  ambiguous[pix] =
 * 1 where a skip / stop decision was within rounding reach of its
 * threshold (the GPU's exp is approximate). */
void oracle_alpha_blending_forward(int P, int C, const float *uv, const float *conic, const float *opacity,
                                   const float *feature, const int32_t *idx_sorted, const int32_t *tile_range,
                                   float bg, int W, int H, float *out, float *final_T, int32_t *ncontrib,
                                   uint8_t *ambiguous) {
    (void)P;
    const int gx = (W + TILE - 1) / TILE;
#ifdef _OPENMP
#pragma omp parallel num_threads(g_threads)
#endif
    {
    float *F = (float *)malloc(sizeof(float) * (C > 0 ? C : 1));
#ifdef _OPENMP
#pragma omp for schedule(static, 1)
#endif
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            const int tile = (py / TILE) * gx + px / TILE;
            const int s = tile_range[2 * tile], e = tile_range[2 * tile + 1];
            float T = 1.0f;
            int last = 0, amb = 0;
            for (int c = 0; c < C; ++c) F[c] = 0;
            for (int j = s; j < e; ++j) {
                const int g = idx_sorted[j];
                const float dx = uv[2 * g] - (float)px, dy = uv[2 * g + 1] - (float)py;
                const float pw = blend_power(conic[3 * g], conic[3 * g + 1], conic[3 * g + 2], dx, dy);
                if (pw > 0.0f) continue;
                const float ex = (float)exp((double)pw);
                const float alpha = fminf(0.99f, opacity[g] * ex);
                if (NEAR(alpha, 1.0f / 255.0f)) amb = 1;
                if (alpha < 1.0f / 255.0f) continue;
                const float nT = T * (1.0f - alpha);
                if (NEAR(nT, 0.0001f)) amb = 1;
                if (nT < 0.0001f) break;
                for (int c = 0; c < C; ++c) F[c] += feature[(size_t)g * C + c] * alpha * T;
                T = nT;
                last = j - s + 1;
            }
            const int pix = py * W + px;
            final_T[pix] = T;
            ncontrib[pix] = last;
            if (ambiguous) ambiguous[pix] = (uint8_t)amb;
            for (int c = 0; c < C; ++c) out[(size_t)c * H * W + pix] = F[c] + T * bg;
        }
    free(F);
    }
}

/* ------------------------------------------------- guided blend replay */
/* The blend makes two threshold decisions per pair: skip when alpha < 1/255,
 * stop when T (1 - alpha) < 1e-4.  The GPU (like the reference's fast-math
 * build) evaluates exp approximately, within a few 1e-7 relative, so an
 * alpha within BLEND_ALPHA_WIN (relative) of 1/255 can land on either side;
 * T is a product of up to hundreds of (1 - alpha) factors, so a T (1 - alpha)
 * within BLEND_T_WIN of 1e-4 can too.  Every other decision is fixed by the
 * float operations, which the oracle reproduces.
 *
 * The guided replay takes a GPU's per-pixel outcome (final T, ncontrib) and
 * finds, per pixel, the path through the list whose flagged decisions take
 * the fewest alternate branches (at most GUIDE_MAX_DEPTH) and whose own
 * outcome matches: the same ncontrib and a final T within BLEND_MATCH
 * (relative).  Taking or skipping a pair changes T by a factor of at least
 * 1 - 1/255 (0.4 %), so the match is unambiguous.  Where no such path
 * exists the pixel is reported unresolved.  Nothing of the GPU's output is
 * copied: the colour, T and ncontrib are the oracle's own along that path. */
#define BLEND_ALPHA_WIN 2e-5f
#define BLEND_T_WIN 1e-3f
#define BLEND_MATCH 1e-3f
#define GUIDE_MAX_DEPTH 3
#define GUIDE_MAX_CAND 48
#define GUIDE_MAX_RUNS 8192

typedef struct {
    int j;    /* list position */
    int kind; /* 0: the alpha >= 1/255 test (take = blend), 1: the T < 1e-4 test (take = stop) */
    int take;
} Decision;

typedef struct {
    const float *uv, *conic, *opacity, *feature;
    const int32_t *idx;
    int s, e, C;
    float px, py;
} PixelList;

static int forced(const Decision *f, int nf, int j, int kind, int dflt) {
    for (int k = 0; k < nf; ++k)
        if (f[k].j == j && f[k].kind == kind) return f[k].take;
    return dflt;
}

/* One front-to-back pass over a pixel's list (msplat/src/alpha_blending.cu:
 * 74-101) with the decisions in `force` replacing the IEEE ones; records the
 * decisions within rounding reach (at most maxc) in cand. */
static void blend_pixel_pass(const PixelList *L, const Decision *force, int nforce, float *F, float *T_out,
                             int *last_out, Decision *cand, int *ncand, int maxc) {
    float T = 1.0f;
    int last = 0, nc = 0;
    for (int c = 0; c < L->C; ++c) F[c] = 0;
    for (int j = L->s; j < L->e; ++j) {
        const int g = L->idx[j];
        const float dx = L->uv[2 * g] - L->px, dy = L->uv[2 * g + 1] - L->py;
        const float pw = blend_power(L->conic[3 * g], L->conic[3 * g + 1], L->conic[3 * g + 2], dx, dy);
        if (pw > 0.0f) continue;
        const float alpha = fminf(0.99f, L->opacity[g] * (float)exp((double)pw));
        int take = !(alpha < 1.0f / 255.0f);
        if (fabsf(alpha - 1.0f / 255.0f) <= BLEND_ALPHA_WIN * (1.0f / 255.0f)) {
            if (nc < maxc) cand[nc] = (Decision){j, 0, take};
            ++nc;
        }
        take = forced(force, nforce, j, 0, take);
        if (!take) continue;
        const float nT = T * (1.0f - alpha);
        int stop = nT < 0.0001f;
        if (fabsf(nT - 0.0001f) <= BLEND_T_WIN * 0.0001f) {
            if (nc < maxc) cand[nc] = (Decision){j, 1, stop};
            ++nc;
        }
        stop = forced(force, nforce, j, 1, stop);
        if (stop) break;
        for (int c = 0; c < L->C; ++c) F[c] += L->feature[(size_t)g * L->C + c] * alpha * T;
        T = nT;
        last = j - L->s + 1;
    }
    *T_out = T;
    *last_out = last;
    *ncand = nc < maxc ? nc : maxc;
}

static int outcome_matches(float T, int last, float gT, int gnc) {
    return last == gnc && fabsf(T - gT) <= BLEND_MATCH * fmaxf(fabsf(T), fabsf(gT));
}

typedef struct {
    const PixelList *L;
    float gT;
    int gnc;
    float *F;
    int runs;
    int found;
    float best_err;
    int best_n;
    Decision best[GUIDE_MAX_DEPTH];
} GuideSearch;

/* Depth-first over flips of flagged decisions after position (j0, kind0),
 * `left` more flips allowed; keeps the matching path with the smallest
 * |T - gT| among those with exactly `left` + nf flips. */
static void guide_dfs(GuideSearch *S, Decision *path, int nf, const Decision *cand, int ncand, int left) {
    for (int k = 0; k < ncand && S->runs < GUIDE_MAX_RUNS; ++k) {
        const Decision c = cand[k];
        if (nf > 0) {
            const Decision p = path[nf - 1];
            if (c.j < p.j || (c.j == p.j && c.kind <= p.kind)) continue;
        }
        path[nf] = (Decision){c.j, c.kind, !c.take};
        float T;
        int last, nc2;
        Decision cand2[GUIDE_MAX_CAND];
        blend_pixel_pass(S->L, path, nf + 1, S->F, &T, &last, cand2, &nc2, GUIDE_MAX_CAND);
        S->runs++;
        if (left == 1) {
            if (outcome_matches(T, last, S->gT, S->gnc)) {
                const float err = fabsf(T - S->gT);
                if (!S->found || err < S->best_err) {
                    S->found = 1;
                    S->best_err = err;
                    S->best_n = nf + 1;
                    for (int q = 0; q <= nf; ++q) S->best[q] = path[q];
                }
            }
        } else {
            guide_dfs(S, path, nf + 1, cand2, nc2, left - 1);
        }
    }
}

/* Guided replay of msplat/src/alpha_blending.cu:16-110 (see above).
 * gpu_T / gpu_ncontrib: the outcome to follow.  Writes the oracle's own out,
 * final_T, ncontrib along the chosen path; nflips[pix] = number of alternate
 * branches taken (0 on the IEEE path), 255 when unresolved; forces[3 pix + k]
 * (k < 3) = the alternate alpha decisions taken, packed j * 2 + take, -1 for
 * none (for oracle_alpha_blending_backward_guided).  Returns the number of
 * unresolved pixels. */
int64_t oracle_alpha_blending_forward_guided(int P, int C, const float *uv, const float *conic,
                                             const float *opacity, const float *feature, const int32_t *idx_sorted,
                                             const int32_t *tile_range, float bg, int W, int H, const float *gpu_T,
                                             const int32_t *gpu_ncontrib, float *out, float *final_T,
                                             int32_t *ncontrib, uint8_t *nflips, int32_t *forces) {
    (void)P;
    const int gx = (W + TILE - 1) / TILE;
    int64_t unresolved = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(g_threads) reduction(+ : unresolved)
#endif
    {
    float *F = (float *)malloc(sizeof(float) * (C > 0 ? C : 1));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            const int tile = (py / TILE) * gx + px / TILE;
            const int pix = py * W + px;
            PixelList L = {uv, conic, opacity, feature, idx_sorted, tile_range[2 * tile], tile_range[2 * tile + 1],
                           C, (float)px, (float)py};
            Decision cand[GUIDE_MAX_CAND], path[GUIDE_MAX_DEPTH];
            float T;
            int last, nc;
            int nfl = 0;
            Decision chosen[GUIDE_MAX_DEPTH];
            blend_pixel_pass(&L, NULL, 0, F, &T, &last, cand, &nc, GUIDE_MAX_CAND);
            int bad = 0;
            if (!outcome_matches(T, last, gpu_T[pix], gpu_ncontrib[pix])) {
                GuideSearch S = {&L, gpu_T[pix], gpu_ncontrib[pix], F, 0, 0, 0.0f, 0, {{0, 0, 0}}};
                for (int d = 1; d <= GUIDE_MAX_DEPTH && !S.found; ++d) guide_dfs(&S, path, 0, cand, nc, d);
                if (S.found) {
                    nfl = S.best_n;
                    for (int d = 0; d < nfl; ++d) chosen[d] = S.best[d];
                    Decision none[1];
                    int n2;
                    blend_pixel_pass(&L, chosen, nfl, F, &T, &last, none, &n2, 0);
                } else {
                    /* unresolved: report the IEEE path */
                    bad = 1;
                    ++unresolved;
                    blend_pixel_pass(&L, NULL, 0, F, &T, &last, cand, &nc, 0);
                }
            }
            final_T[pix] = T;
            ncontrib[pix] = last;
            if (nflips) nflips[pix] = (uint8_t)(bad ? 255 : nfl);
            if (forces) {
                int k = 0;
                for (int d = 0; d < nfl; ++d)
                    if (chosen[d].kind == 0 && k < 3) forces[3 * (size_t)pix + k++] = chosen[d].j * 2 + chosen[d].take;
                for (; k < 3; ++k) forces[3 * (size_t)pix + k] = -1;
            }
            for (int c = 0; c < C; ++c) out[(size_t)c * H * W + pix] = F[c] + T * bg;
        }
    free(F);
    }
    return unresolved;
}

/* msplat/src/alpha_blending.cu:112-246, in double given the forward's
 * final_T / ncontrib.  Gradients are written (zero-filled first). */
static void blend_backward_impl(int P, int C, const float *uv, const float *conic, const float *opacity,
                                const float *feature, const int32_t *idx_sorted, const int32_t *tile_range,
                                float bg, int W, int H, const float *final_T, const int32_t *ncontrib,
                                const float *dL_dout, const int32_t *forces, double *dL_duv, double *dL_dconic,
                                double *dL_dop, double *dL_dfeat) {
    const int gx = (W + TILE - 1) / TILE;
    memset(dL_duv, 0, sizeof(double) * 2 * (size_t)P);
    memset(dL_dconic, 0, sizeof(double) * 3 * (size_t)P);
    memset(dL_dop, 0, sizeof(double) * (size_t)P);
    memset(dL_dfeat, 0, sizeof(double) * (size_t)P * C);
    /* Thread 0 accumulates into the outputs; threads 1.. into private
     * buffers that are added afterwards in thread order. */
    const size_t per = (size_t)P * (6 + C);
    double *priv = g_threads > 1 ? (double *)calloc(per * (size_t)(g_threads - 1), sizeof(double)) : NULL;
    int nteam = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(g_threads)
#endif
    {
    const int tid = thread_id();
    if (tid == 0) nteam = team_size();
    double *dL_duv_t = dL_duv, *dL_dconic_t = dL_dconic, *dL_dop_t = dL_dop, *dL_dfeat_t = dL_dfeat;
    if (tid > 0) {
        double *b = priv + per * (size_t)(tid - 1);
        dL_duv_t = b;
        dL_dconic_t = b + 2 * (size_t)P;
        dL_dop_t = b + 5 * (size_t)P;
        dL_dfeat_t = b + 6 * (size_t)P;
    }
    double *acc = (double *)malloc(sizeof(double) * 3 * (C > 0 ? C : 1));
    double *lastf = acc + C, *dpix = acc + 2 * C;
#ifdef _OPENMP
#pragma omp for schedule(static, 1)
#endif
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            const int tile = (py / TILE) * gx + px / TILE;
            const int s = tile_range[2 * tile];
            const int pix = py * W + px;
            const double Tf = final_T[pix];
            const int last = ncontrib[pix];
            double T = Tf, last_alpha = 0, bg_dot = 0;
            for (int c = 0; c < C; ++c) {
                acc[c] = 0;
                lastf[c] = 0;
                dpix[c] = dL_dout[(size_t)c * H * W + pix];
                bg_dot += bg * dpix[c];
            }
            for (int j = s + last - 1; j >= s; --j) {
                const int g = idx_sorted[j];
                const double dx = (double)uv[2 * g] - px, dy = (double)uv[2 * g + 1] - py;
                const double a = conic[3 * g], b = conic[3 * g + 1], c_ = conic[3 * g + 2];
                const double pw = -0.5 * (a * dx * dx + c_ * dy * dy) - b * dx * dy;
                if (forces) {
                    /* the forward's float decisions, with its alternate
                     * branches (guided replay) */
                    const float pwf = blend_power(conic[3 * g], conic[3 * g + 1], conic[3 * g + 2],
                                                  uv[2 * g] - (float)px, uv[2 * g + 1] - (float)py);
                    if (pwf > 0.0f) continue;
                    const float af = fminf(0.99f, opacity[g] * (float)exp((double)pwf));
                    int take = !(af < 1.0f / 255.0f);
                    for (int k = 0; k < 3; ++k) {
                        const int32_t f = forces[3 * (size_t)pix + k];
                        if (f >= 0 && f / 2 == j) take = f & 1;
                    }
                    if (!take) continue;
                } else if (pw > 0) {
                    continue;
                }
                const double G = exp(pw);
                const double op = opacity[g];
                const double alpha = fmin(0.99, op * G);
                if (!forces && alpha < 1.0 / 255.0) continue;
                T = T / (1.0 - alpha);
                const double dcol = alpha * T;
                double dL_dalpha = 0;
                for (int c = 0; c < C; ++c) {
                    const double f = feature[(size_t)g * C + c];
                    acc[c] = last_alpha * lastf[c] + (1.0 - last_alpha) * acc[c];
                    lastf[c] = f;
                    dL_dalpha += (f - acc[c]) * dpix[c];
                    dL_dfeat_t[(size_t)g * C + c] += dcol * dpix[c];
                }
                dL_dalpha *= T;
                last_alpha = alpha;
                dL_dalpha += (-Tf / (1.0 - alpha)) * bg_dot;
                const double dG = op * dL_dalpha;
                dL_duv_t[2 * g] += dG * (-G * dx * a - G * dy * b);
                dL_duv_t[2 * g + 1] += dG * (-G * dy * c_ - G * dx * b);
                dL_dconic_t[3 * g] += -0.5 * G * dx * dx * dG;
                dL_dconic_t[3 * g + 1] += -G * dx * dy * dG;
                dL_dconic_t[3 * g + 2] += -0.5 * G * dy * dy * dG;
                dL_dop_t[g] += G * dL_dalpha;
            }
        }
    free(acc);
    }
    if (priv) {
        PARFOR
        for (int g = 0; g < P; ++g)
            for (int t = 1; t < nteam; ++t) {
                const double *b = priv + per * (size_t)(t - 1);
                dL_duv[2 * g] += b[2 * (size_t)g];
                dL_duv[2 * g + 1] += b[2 * (size_t)g + 1];
                for (int k = 0; k < 3; ++k) dL_dconic[3 * g + k] += b[2 * (size_t)P + 3 * (size_t)g + k];
                dL_dop[g] += b[5 * (size_t)P + g];
                for (int c = 0; c < C; ++c) dL_dfeat[(size_t)g * C + c] += b[6 * (size_t)P + (size_t)g * C + c];
            }
        free(priv);
    }
}

void oracle_alpha_blending_backward(int P, int C, const float *uv, const float *conic, const float *opacity,
                                    const float *feature, const int32_t *idx_sorted, const int32_t *tile_range,
                                    float bg, int W, int H, const float *final_T, const int32_t *ncontrib,
                                    const float *dL_dout, double *dL_duv, double *dL_dconic, double *dL_dop,
                                    double *dL_dfeat) {
    blend_backward_impl(P, C, uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, final_T, ncontrib,
                        dL_dout, NULL, dL_duv, dL_dconic, dL_dop, dL_dfeat);
}

/* The backward along the paths of oracle_alpha_blending_forward_guided:
 * the skip decisions are the forward's float ones with its alternate
 * branches (`forces`), so the pairs differentiated are those the GPU
 * blended. */
void oracle_alpha_blending_backward_guided(int P, int C, const float *uv, const float *conic,
                                           const float *opacity, const float *feature, const int32_t *idx_sorted,
                                           const int32_t *tile_range, float bg, int W, int H, const float *final_T,
                                           const int32_t *ncontrib, const float *dL_dout, const int32_t *forces,
                                           double *dL_duv, double *dL_dconic, double *dL_dop, double *dL_dfeat) {
    blend_backward_impl(P, C, uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, final_T, ncontrib,
                        dL_dout, forces, dL_duv, dL_dconic, dL_dop, dL_dfeat);
}
