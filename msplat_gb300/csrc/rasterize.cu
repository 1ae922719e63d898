// Fused per-Gaussian preprocessing of a rasterisation: projection, 3-D
// covariance, EWA splat (and optionally SH colour from view directions) in
// one forward kernel, and all of their adjoints -- including the camera
// (intrinsics / extrinsics) gradients -- in one backward kernel.
//
// This is the composite of msplat/__init__.py:70-93 (project_point ->
// compute_cov3d -> ewa_project) plus the view-direction SH colour that the
// reference's training loops evaluate before calling it.  Every quantity
// comes from the same device functions as the single-stage kernels
// (geometry.cuh), so uv, depth, conic, radius and tiles are bit-identical
// to the stage-by-stage path; the covariance is recomputed in the backward
// instead of being stored.
#include "geometry.cuh"
#include "sh_basis.cuh"
#include "sh_dispatch.cuh"

namespace msplat {

__global__ void __launch_bounds__(256)
preprocess_fwd_kernel(int P, const float *__restrict__ xyz, const float *__restrict__ scales,
                      const float4 *__restrict__ quats, const float *__restrict__ intr,
                      const float *__restrict__ extr, int W, int H, float nearest, float extent, int gx, int gy,
                      float2 *__restrict__ uv, float *__restrict__ depth, float *__restrict__ conic,
                      int32_t *__restrict__ radius, int32_t *__restrict__ tiles) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const Cam c = load_cam(intr, extr);
    const float px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
    float2 u;
    float d;
    project_fwd_one(c, px, py, pz, W, H, nearest, extent, u, d);
    uv[i] = u;
    depth[i] = d;
    float o[3] = {0.f, 0.f, 0.f};
    int rad = 0, nt = 0;
    if (d != 0.0f) {  // visible = depth != 0, as the reference's rasterization
        float cov[6];
        cov3d_fwd_one(scales[3 * i], scales[3 * i + 1], scales[3 * i + 2], quats[i], cov);
        ewa_fwd_one(c, px, py, pz, cov, u, gx, gy, o, rad, nt);
    }
    conic[3 * i + 0] = o[0];
    conic[3 * i + 1] = o[1];
    conic[3 * i + 2] = o[2];
    radius[i] = rad;
    tiles[i] = nt;
}

// Geometry and view-direction SH colour in one kernel (SH degree <= 3,
// C <= 4, the common case): the block's coefficient rows are staged in
// shared memory as sh_fwd_kernel stages them, the geometry of
// preprocess_fwd_kernel runs while those loads are in flight, and the
// colour follows with sh_fwd_kernel's code (camera-centre view direction,
// the same products in the same order), so every output is identical to
// the two-kernel path.
template <int DEG>
__global__ void __launch_bounds__(256)
preprocess_sh_fwd_kernel(int P, int C, const float *__restrict__ xyz, const float *__restrict__ scales,
                         const float4 *__restrict__ quats, const float *__restrict__ intr,
                         const float *__restrict__ extr, int W, int H, float nearest, float extent, int gx, int gy,
                         const float *__restrict__ shs, float2 *__restrict__ uv, float *__restrict__ depth,
                         float *__restrict__ conic, int32_t *__restrict__ radius, int32_t *__restrict__ tiles,
                         float *__restrict__ color) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    extern __shared__ float smem[];
    const int CD = C * D, stride = CD | 1;
    const int p0 = blockIdx.x * blockDim.x;
    const int n = min((int)blockDim.x, P - p0);
    stage_rows(smem, shs + (size_t)p0 * CD, n, CD, stride);
    const int t = threadIdx.x;
    const int i = p0 + t;
    float px = 0.f, py = 0.f, pz = 0.f, d = 0.f;
    if (t < n) {
        const Cam c = load_cam(intr, extr);
        px = xyz[3 * i];
        py = xyz[3 * i + 1];
        pz = xyz[3 * i + 2];
        float2 u;
        project_fwd_one(c, px, py, pz, W, H, nearest, extent, u, d);
        uv[i] = u;
        depth[i] = d;
        float o[3] = {0.f, 0.f, 0.f};
        int rad = 0, nt = 0;
        if (d != 0.0f) {  // visible = depth != 0, as the reference's rasterization
            float cov[6];
            cov3d_fwd_one(scales[3 * i], scales[3 * i + 1], scales[3 * i + 2], quats[i], cov);
            ewa_fwd_one(c, px, py, pz, cov, u, gx, gy, o, rad, nt);
        }
        conic[3 * i + 0] = o[0];
        conic[3 * i + 1] = o[1];
        conic[3 * i + 2] = o[2];
        radius[i] = rad;
        tiles[i] = nt;
    }
    __syncthreads();
    if (t >= n) return;
    float *out = color + (size_t)i * C;
    if (d == 0.0f) {
        for (int ch = 0; ch < C; ++ch) out[ch] = 0.f;
        return;
    }
    float cc[3];
    camera_centre(extr, cc);
    const float dx = px - cc[0], dy = py - cc[1], dz = pz - cc[2];
    const float len = sqrtf(dx * dx + dy * dy + dz * dz);
    const float vx = dx / len, vy = dy / len, vz = dz / len;
    const float *row = smem + t * stride;
    for (int c0 = 0; c0 < C; c0 += kShChanBlock) {
        float acc[kShChanBlock] = {0.f, 0.f, 0.f, 0.f};
        const int nc = min(kShChanBlock, C - c0);
        sh_basis<DEG, false>(vx, vy, vz, [&](int k, float Y) {
#pragma unroll
            for (int cb = 0; cb < kShChanBlock; ++cb)
                if (cb < nc) acc[cb] += Y * row[(c0 + cb) * D + k];
        });
        for (int cb = 0; cb < nc; ++cb) out[c0 + cb] = acc[cb];
    }
}

// dL/dxyz accumulates (projection + EWA) onto what the SH backward wrote
// there when add_xyz is set.  That value gv is the adjoint of the view
// direction's v = x - c, so the camera centre c = -R^T T receives -gv:
// dL/dR(r,j) += T_r gv_j and dL/dT_r += sum_j R(r,j) gv_j.
// 3 blocks per SM: 80 registers (a 24-byte spill) instead of 120.
__global__ void __launch_bounds__(256, 3)
preprocess_bwd_kernel(int P, const float *__restrict__ xyz, const float *__restrict__ scales,
                      const float4 *__restrict__ quats, const float *__restrict__ intr,
                      const float *__restrict__ extr, const float *__restrict__ depth,
                      const int32_t *__restrict__ radius, const float2 *__restrict__ dL_duv,
                      const float *__restrict__ dL_dconic, bool add_xyz, float *dL_dxyz,
                      float *__restrict__ dL_dscales, float4 *__restrict__ dL_dquats, bool cam_grads,
                      float *__restrict__ partials) {
    const Cam c = load_cam(intr, extr);
    float acc[kCamGradVals];
#pragma unroll
    for (int k = 0; k < kCamGradVals; ++k) acc[k] = 0.0f;

    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        float g[3] = {0.f, 0.f, 0.f};
        float ds[3] = {0.f, 0.f, 0.f};
        float4 dq = make_float4(0.f, 0.f, 0.f, 0.f);
        if (depth[i] != 0.0f) {
            const float px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
            project_bwd_one(c, px, py, pz, dL_duv[i], 0.0f, g, cam_grads, acc);
            if (radius[i] > 0) {
                const float s[3] = {scales[3 * i], scales[3 * i + 1], scales[3 * i + 2]};
                const float4 q = quats[i];
                float cov[6], ge[3], dV[6];
                cov3d_fwd_one(s[0], s[1], s[2], q, cov);
                if (ewa_bwd_one(c, px, py, pz, cov, dL_dconic[3 * i], dL_dconic[3 * i + 1], dL_dconic[3 * i + 2],
                                ge, dV, cam_grads, acc)) {
                    cov3d_bwd_one(s, q, dV, ds, dq);
#pragma unroll
                    for (int k = 0; k < 3; ++k) g[k] += ge[k];
                }
            }
        }
        if (add_xyz) {
            const float gv[3] = {dL_dxyz[3 * i], dL_dxyz[3 * i + 1], dL_dxyz[3 * i + 2]};
#pragma unroll
            for (int k = 0; k < 3; ++k) g[k] += gv[k];
            if (cam_grads) {
#pragma unroll
                for (int r = 0; r < 3; ++r) {
#pragma unroll
                    for (int j = 0; j < 3; ++j) acc[4 + 4 * r + j] += c.e[4 * r + 3] * gv[j];
                    acc[4 + 4 * r + 3] += c.e[4 * r] * gv[0] + c.e[4 * r + 1] * gv[1] + c.e[4 * r + 2] * gv[2];
                }
            }
        }
        dL_dxyz[3 * i + 0] = g[0];
        dL_dxyz[3 * i + 1] = g[1];
        dL_dxyz[3 * i + 2] = g[2];
        dL_dscales[3 * i + 0] = ds[0];
        dL_dscales[3 * i + 1] = ds[1];
        dL_dscales[3 * i + 2] = ds[2];
        dL_dquats[i] = dq;
    }
    if (cam_grads) block_partial_16(acc, partials);
}

// The SH adjoint and the geometry adjoint in one kernel (SH degree <= 3,
// C <= 4): each step of preprocess_bwd_kernel's loop stages its block's
// coefficient rows as sh_bwd_kernel does, evaluates the SH adjoint in
// place (dL/dsh) and its view-direction gradient gv, then runs the
// geometry adjoint with gv in registers instead of reading it back from
// dL/dxyz, and streams the dL/dsh rows out.  The same Gaussians go to the
// same threads in the same order, and every sum is taken in the same
// order as in the two-kernel path, so all outputs are identical.
template <int DEG>
__global__ void __launch_bounds__(256, 3)
preprocess_sh_bwd_kernel(int P, int C, const float *__restrict__ xyz, const float *__restrict__ scales,
                         const float4 *__restrict__ quats, const float *__restrict__ intr,
                         const float *__restrict__ extr, const float *__restrict__ shs,
                         const float *__restrict__ depth, const int32_t *__restrict__ radius,
                         const float2 *__restrict__ dL_duv, const float *__restrict__ dL_dconic,
                         const float *__restrict__ dL_dcolor, float *__restrict__ dL_dxyz,
                         float *__restrict__ dL_dscales, float4 *__restrict__ dL_dquats, float *__restrict__ dL_dshs,
                         bool cam_grads, float *__restrict__ partials) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    extern __shared__ float smem[];
    const int CD = C * D, stride = CD | 1;
    const Cam c = load_cam(intr, extr);
    float cc[3];
    camera_centre(extr, cc);
    float acc[kCamGradVals];
#pragma unroll
    for (int k = 0; k < kCamGradVals; ++k) acc[k] = 0.0f;
    const int t = threadIdx.x;
    for (int p0 = blockIdx.x * blockDim.x; p0 < P; p0 += gridDim.x * blockDim.x) {
        const int n = min((int)blockDim.x, P - p0);
        stage_rows(smem, shs + (size_t)p0 * CD, n, CD, stride);
        __syncthreads();
        if (t < n) {
            const int i = p0 + t;
            float *row = smem + t * stride;
            const float px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
            const float dep = depth[i];
            // SH adjoint (sh_bwd_kernel, camera mode)
            float gv[3] = {0.f, 0.f, 0.f};
            if (dep == 0.0f) {
                for (int k = 0; k < CD; ++k) row[k] = 0.f;
            } else {
                const float dx = px - cc[0], dy = py - cc[1], dz = pz - cc[2];
                const float len = sqrtf(dx * dx + dy * dy + dz * dz);
                const float d[3] = {dx / len, dy / len, dz / len};
                float gdx = 0.f, gdy = 0.f, gdz = 0.f;
                for (int c0 = 0; c0 < C; c0 += kShChanBlock) {
                    float g[kShChanBlock] = {0.f, 0.f, 0.f, 0.f};
                    const int nc = min(kShChanBlock, C - c0);
                    for (int cb = 0; cb < nc; ++cb) g[cb] = dL_dcolor[(size_t)i * C + c0 + cb];
                    sh_basis<DEG, true>(d[0], d[1], d[2], [&](int k, float Y, float yx, float yy, float yz) {
#pragma unroll
                        for (int cb = 0; cb < kShChanBlock; ++cb) {
                            if (cb < nc) {
                                float *slot = row + (c0 + cb) * D + k;
                                const float w = g[cb] * *slot;  // dL/dval * coefficient
                                gdx += w * yx;
                                gdy += w * yy;
                                gdz += w * yz;
                                *slot = g[cb] * Y;  // dL/dsh, written in place
                            }
                        }
                    });
                }
                const float dg = d[0] * gdx + d[1] * gdy + d[2] * gdz;
                gv[0] = (gdx - d[0] * dg) / len;
                gv[1] = (gdy - d[1] * dg) / len;
                gv[2] = (gdz - d[2] * dg) / len;
            }
            // geometry adjoint (preprocess_bwd_kernel with add_xyz)
            float gx3[3] = {0.f, 0.f, 0.f};
            float ds[3] = {0.f, 0.f, 0.f};
            float4 dq = make_float4(0.f, 0.f, 0.f, 0.f);
            if (dep != 0.0f) {
                project_bwd_one(c, px, py, pz, dL_duv[i], 0.0f, gx3, cam_grads, acc);
                if (radius[i] > 0) {
                    const float s3[3] = {scales[3 * i], scales[3 * i + 1], scales[3 * i + 2]};
                    const float4 q = quats[i];
                    float cov[6], ge[3], dV[6];
                    cov3d_fwd_one(s3[0], s3[1], s3[2], q, cov);
                    if (ewa_bwd_one(c, px, py, pz, cov, dL_dconic[3 * i], dL_dconic[3 * i + 1], dL_dconic[3 * i + 2],
                                    ge, dV, cam_grads, acc)) {
                        cov3d_bwd_one(s3, q, dV, ds, dq);
#pragma unroll
                        for (int k = 0; k < 3; ++k) gx3[k] += ge[k];
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) gx3[k] += gv[k];
            if (cam_grads) {
#pragma unroll
                for (int r = 0; r < 3; ++r) {
#pragma unroll
                    for (int j = 0; j < 3; ++j) acc[4 + 4 * r + j] += c.e[4 * r + 3] * gv[j];
                    acc[4 + 4 * r + 3] += c.e[4 * r] * gv[0] + c.e[4 * r + 1] * gv[1] + c.e[4 * r + 2] * gv[2];
                }
            }
            dL_dxyz[3 * i + 0] = gx3[0];
            dL_dxyz[3 * i + 1] = gx3[1];
            dL_dxyz[3 * i + 2] = gx3[2];
            dL_dscales[3 * i + 0] = ds[0];
            dL_dscales[3 * i + 1] = ds[1];
            dL_dscales[3 * i + 2] = ds[2];
            dL_dquats[i] = dq;
        }
        __syncthreads();
        unstage_rows(dL_dshs + (size_t)p0 * CD, smem, n, CD, stride);
        __syncthreads();  // the rows are staged again by the next step
    }
    if (cam_grads) block_partial_16(acc, partials);
}

// ---- three channels, rows of whole 16-byte vectors (degrees 1 and 3) ------
// The common RGB case without shared memory: each thread reads its own
// Gaussian's coefficient row (3 D floats, D a multiple of 4, the array
// 16-byte aligned) straight into registers with 16-byte streaming loads,
// all issued before anything else, so every resident thread has its whole
// row in flight and no block waits at a barrier for a staging loop.  The
// arithmetic, its order and the outputs are those of
// preprocess_sh_fwd_kernel / preprocess_sh_bwd_kernel for C = 3.
#ifndef MSPLAT_PREP_ROWREG
#define MSPLAT_PREP_ROWREG 1
#endif

template <int CD>
__device__ __forceinline__ void load_row_regs(const float *__restrict__ shs, int i, float (&r)[CD]) {
    const float4 *src = reinterpret_cast<const float4 *>(shs) + (size_t)i * (CD / 4);
#pragma unroll
    for (int u = 0; u < CD / 4; ++u) {
        const float4 q = __ldcs(src + u);
        r[4 * u] = q.x;
        r[4 * u + 1] = q.y;
        r[4 * u + 2] = q.z;
        r[4 * u + 3] = q.w;
    }
}

// 3 blocks per SM: 80 registers (a 4-byte spill) instead of 92.
template <int DEG>
__global__ void __launch_bounds__(256, 3)
preprocess_sh3_fwd_kernel(int P, const float *__restrict__ xyz, const float *__restrict__ scales,
                          const float4 *__restrict__ quats, const float *__restrict__ intr,
                          const float *__restrict__ extr, int W, int H, float nearest, float extent, int gx, int gy,
                          const float *__restrict__ shs, float2 *__restrict__ uv, float *__restrict__ depth,
                          float *__restrict__ conic, int32_t *__restrict__ radius, int32_t *__restrict__ tiles,
                          float *__restrict__ color) {
    constexpr int D = (DEG + 1) * (DEG + 1), CD = 3 * D;
    static_assert(CD % 4 == 0, "rows of whole 16-byte vectors");
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    float r[CD];
    load_row_regs<CD>(shs, i, r);
    const Cam c = load_cam(intr, extr);
    const float px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
    float2 u;
    float d;
    project_fwd_one(c, px, py, pz, W, H, nearest, extent, u, d);
    uv[i] = u;
    depth[i] = d;
    float o[3] = {0.f, 0.f, 0.f};
    int rad = 0, nt = 0;
    if (d != 0.0f) {  // visible = depth != 0, as the reference's rasterization
        float cov[6];
        cov3d_fwd_one(scales[3 * i], scales[3 * i + 1], scales[3 * i + 2], quats[i], cov);
        ewa_fwd_one(c, px, py, pz, cov, u, gx, gy, o, rad, nt);
    }
    conic[3 * i + 0] = o[0];
    conic[3 * i + 1] = o[1];
    conic[3 * i + 2] = o[2];
    radius[i] = rad;
    tiles[i] = nt;
    float *out = color + (size_t)i * 3;
    if (d == 0.0f) {
        out[0] = out[1] = out[2] = 0.f;
        return;
    }
    float cc[3];
    camera_centre(extr, cc);
    const float dx = px - cc[0], dy = py - cc[1], dz = pz - cc[2];
    const float len = sqrtf(dx * dx + dy * dy + dz * dz);
    const float vx = dx / len, vy = dy / len, vz = dz / len;
    float acc[3] = {0.f, 0.f, 0.f};
    sh_basis<DEG, false>(vx, vy, vz, [&](int k, float Y) {
#pragma unroll
        for (int cb = 0; cb < 3; ++cb) acc[cb] += Y * r[cb * D + k];
    });
    out[0] = acc[0];
    out[1] = acc[1];
    out[2] = acc[2];
}

template <int DEG>
__global__ void __launch_bounds__(256, 2)
preprocess_sh3_bwd_kernel(int P, const float *__restrict__ xyz, const float *__restrict__ scales,
                          const float4 *__restrict__ quats, const float *__restrict__ intr,
                          const float *__restrict__ extr, const float *__restrict__ shs,
                          const float *__restrict__ depth, const int32_t *__restrict__ radius,
                          const float2 *__restrict__ dL_duv, const float *__restrict__ dL_dconic,
                          const float *__restrict__ dL_dcolor, float *__restrict__ dL_dxyz,
                          float *__restrict__ dL_dscales, float4 *__restrict__ dL_dquats,
                          float *__restrict__ dL_dshs, bool cam_grads, float *__restrict__ partials) {
    constexpr int D = (DEG + 1) * (DEG + 1), CD = 3 * D;
    static_assert(CD % 4 == 0, "rows of whole 16-byte vectors");
    const Cam c = load_cam(intr, extr);
    float cc[3];
    camera_centre(extr, cc);
    float acc[kCamGradVals];
#pragma unroll
    for (int k = 0; k < kCamGradVals; ++k) acc[k] = 0.0f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        float r[CD];
        load_row_regs<CD>(shs, i, r);
        const float px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
        const float dep = depth[i];
        const float g[3] = {dL_dcolor[3 * i], dL_dcolor[3 * i + 1], dL_dcolor[3 * i + 2]};
        // SH adjoint (sh_bwd_kernel, camera mode): dL/dsh in place of the row
        float gv[3] = {0.f, 0.f, 0.f};
        if (dep == 0.0f) {
#pragma unroll
            for (int k = 0; k < CD; ++k) r[k] = 0.f;
        } else {
            const float dx = px - cc[0], dy = py - cc[1], dz = pz - cc[2];
            const float len = sqrtf(dx * dx + dy * dy + dz * dz);
            const float d[3] = {dx / len, dy / len, dz / len};
            float gdx = 0.f, gdy = 0.f, gdz = 0.f;
            sh_basis<DEG, true>(d[0], d[1], d[2], [&](int k, float Y, float yx, float yy, float yz) {
#pragma unroll
                for (int cb = 0; cb < 3; ++cb) {
                    const float w = g[cb] * r[cb * D + k];  // dL/dval * coefficient
                    gdx += w * yx;
                    gdy += w * yy;
                    gdz += w * yz;
                    r[cb * D + k] = g[cb] * Y;  // dL/dsh
                }
            });
            const float dg = d[0] * gdx + d[1] * gdy + d[2] * gdz;
            gv[0] = (gdx - d[0] * dg) / len;
            gv[1] = (gdy - d[1] * dg) / len;
            gv[2] = (gdz - d[2] * dg) / len;
        }
        float4 *dst = reinterpret_cast<float4 *>(dL_dshs) + (size_t)i * (CD / 4);
#pragma unroll
        for (int u = 0; u < CD / 4; ++u) __stcs(dst + u, make_float4(r[4 * u], r[4 * u + 1], r[4 * u + 2], r[4 * u + 3]));
        // geometry adjoint (preprocess_bwd_kernel with add_xyz)
        float gx3[3] = {0.f, 0.f, 0.f};
        float ds[3] = {0.f, 0.f, 0.f};
        float4 dq = make_float4(0.f, 0.f, 0.f, 0.f);
        if (dep != 0.0f) {
            project_bwd_one(c, px, py, pz, dL_duv[i], 0.0f, gx3, cam_grads, acc);
            if (radius[i] > 0) {
                const float s3[3] = {scales[3 * i], scales[3 * i + 1], scales[3 * i + 2]};
                const float4 q = quats[i];
                float cov[6], ge[3], dV[6];
                cov3d_fwd_one(s3[0], s3[1], s3[2], q, cov);
                if (ewa_bwd_one(c, px, py, pz, cov, dL_dconic[3 * i], dL_dconic[3 * i + 1], dL_dconic[3 * i + 2],
                                ge, dV, cam_grads, acc)) {
                    cov3d_bwd_one(s3, q, dV, ds, dq);
#pragma unroll
                    for (int k = 0; k < 3; ++k) gx3[k] += ge[k];
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) gx3[k] += gv[k];
        if (cam_grads) {
#pragma unroll
            for (int rr = 0; rr < 3; ++rr) {
#pragma unroll
                for (int j = 0; j < 3; ++j) acc[4 + 4 * rr + j] += c.e[4 * rr + 3] * gv[j];
                acc[4 + 4 * rr + 3] += c.e[4 * rr] * gv[0] + c.e[4 * rr + 1] * gv[1] + c.e[4 * rr + 2] * gv[2];
            }
        }
        dL_dxyz[3 * i + 0] = gx3[0];
        dL_dxyz[3 * i + 1] = gx3[1];
        dL_dxyz[3 * i + 2] = gx3[2];
        dL_dscales[3 * i + 0] = ds[0];
        dL_dscales[3 * i + 1] = ds[1];
        dL_dscales[3 * i + 2] = ds[2];
        dL_dquats[i] = dq;
    }
    if (cam_grads) block_partial_16(acc, partials);
}

// Whether the register-row kernels take a call: three channels, degree 1
// or 3, every row array 16-byte aligned.
inline bool prep_rowreg(int C, int D, const void *shs, const void *dL_dshs) {
    return MSPLAT_PREP_ROWREG && C == 3 && (D == 4 || D == 16) && ((uintptr_t)shs & 15) == 0 &&
           ((uintptr_t)dL_dshs & 15) == 0;
}

inline int preprocess_bwd_blocks(int P) { return min(ceil_div(P, 256), kCamGradBlocks); }

}  // namespace msplat

using namespace msplat;

extern "C" size_t msplat_rasterize_preprocess_workspace_size(int P, int C, int D) {
    (void)C;
    (void)D;
    if (P <= 0) return 0;
    return (size_t)preprocess_bwd_blocks(P) * kCamGradVals * sizeof(float);
}

extern "C" int msplat_rasterize_preprocess_forward(int P, const float *xyz, const float *scales,
                                                   const float *uquats, const float *intr, const float *extr,
                                                   int W, int H, float nearest, float extent, int C, int D,
                                                   const float *shs, float *uv, float *depth, float *conic,
                                                   int32_t *radius, int32_t *tiles, float *color,
                                                   msplat_stream_t stream) {
    if (P < 0 || W <= 0 || H <= 0 || C < 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "rasterize_preprocess_forward: bad sizes P=%d W=%d H=%d C=%d",
                         P, W, H, C);
    if (P == 0) return MSPLAT_OK;
    if (!xyz || !scales || !uquats || !intr || !extr || !uv || !depth || !conic || !radius || !tiles)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "rasterize_preprocess_forward: null pointer");
    if (((uintptr_t)uquats & 15) != 0 || ((uintptr_t)uv & 7) != 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "rasterize_preprocess_forward: misaligned uquats / uv");
    const bool sh = shs != nullptr && C > 0;
    if (sh && !color)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "rasterize_preprocess_forward: shs given without color");
    const int gx = ceil_div(W, kTile), gy = ceil_div(H, kTile);
    if (sh && prep_rowreg(C, D, shs, nullptr)) {  // one kernel, rows in registers
        if (D == 4)
            launch(preprocess_sh3_fwd_kernel<1>, ceil_div(P, 256), 256, 0, stream, P, xyz, scales,
                   (const float4 *)uquats, intr, extr, W, H, nearest, extent, gx, gy, shs, (float2 *)uv, depth, conic,
                   radius, tiles, color);
        else
            launch(preprocess_sh3_fwd_kernel<3>, ceil_div(P, 256), 256, 0, stream, P, xyz, scales,
                   (const float4 *)uquats, intr, extr, W, H, nearest, extent, gx, gy, shs, (float2 *)uv, depth, conic,
                   radius, tiles, color);
        return check_launch("rasterize_preprocess_forward");
    }
    if (sh && D <= 16 && C <= kShChanBlock) {  // one kernel: geometry and colour
        const size_t smem = (size_t)256 * ((C * D) | 1) * sizeof(float);
#define MSPLAT_PREP_SH(DG)                                                                                       \
    case (DG + 1) * (DG + 1):                                                                                    \
        cudaFuncSetAttribute(preprocess_sh_fwd_kernel<DG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        launch(preprocess_sh_fwd_kernel<DG>, ceil_div(P, 256), 256, smem, stream, P, C, xyz, scales,             \
               (const float4 *)uquats, intr, extr, W, H, nearest, extent, gx, gy, shs, (float2 *)uv, depth, conic, \
               radius, tiles, color);                                                                            \
        return check_launch("rasterize_preprocess_forward");
        switch (D) {
            MSPLAT_PREP_SH(0) MSPLAT_PREP_SH(1) MSPLAT_PREP_SH(2) MSPLAT_PREP_SH(3)
            default: break;
        }
#undef MSPLAT_PREP_SH
    }
    launch(preprocess_fwd_kernel, ceil_div(P, 256), 256, 0, stream, P, xyz, scales, (const float4 *)uquats, intr,
           extr, W, H, nearest, extent, gx, gy, (float2 *)uv, depth, conic, radius, tiles);
    int st = check_launch("rasterize_preprocess_forward");
    if (st || !sh) return st;
    const ShDirs in{nullptr, nullptr, xyz, extr, depth, nullptr};
    return sh_dispatch(false, P, C, D, shs, in, nullptr, color, nullptr, stream);
}

extern "C" int msplat_rasterize_preprocess_backward(
    int P, const float *xyz, const float *scales, const float *uquats, const float *intr, const float *extr,
    int C, int D, const float *shs, const float *depth, const int32_t *radius, const float *dL_duv,
    const float *dL_dconic, const float *dL_dcolor, float *dL_dxyz, float *dL_dscales, float *dL_duquats,
    float *dL_dshs, float *dL_dintr, float *dL_dextr, void *workspace, size_t workspace_bytes,
    msplat_stream_t stream) {
    if (P < 0 || C < 0) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "rasterize_preprocess_backward: bad sizes");
    const bool cam = dL_dintr || dL_dextr;
    if (P == 0) {
        if (dL_dintr) cudaMemsetAsync(dL_dintr, 0, 4 * sizeof(float), stream);
        if (dL_dextr) cudaMemsetAsync(dL_dextr, 0, 12 * sizeof(float), stream);
        return check_launch("rasterize_preprocess_backward");
    }
    if (!xyz || !scales || !uquats || !intr || !extr || !depth || !radius || !dL_duv || !dL_dconic || !dL_dxyz ||
        !dL_dscales || !dL_duquats)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "rasterize_preprocess_backward: null pointer");
    if ((((uintptr_t)uquats | (uintptr_t)dL_duquats) & 15) != 0 || ((uintptr_t)dL_duv & 7) != 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "rasterize_preprocess_backward: misaligned buffers");
    const bool sh = shs != nullptr && C > 0;
    if (sh && (!dL_dcolor || !dL_dshs))
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "rasterize_preprocess_backward: shs without dL_dcolor / dL_dshs");
    const size_t need = msplat_rasterize_preprocess_workspace_size(P, sh ? C : 0, sh ? D : 0);
    if (cam && (!workspace || workspace_bytes < need))
        return set_error(MSPLAT_ERR_WORKSPACE, "rasterize_preprocess_backward: workspace of %zu bytes < %zu",
                         workspace_bytes, need);
    const int gblocks = preprocess_bwd_blocks(P);
    float *partials = (float *)workspace;
    if (sh && prep_rowreg(C, D, shs, dL_dshs)) {  // one kernel, rows in registers
        if (D == 4)
            launch(preprocess_sh3_bwd_kernel<1>, gblocks, 256, 0, stream, P, xyz, scales, (const float4 *)uquats, intr,
                   extr, shs, depth, radius, (const float2 *)dL_duv, dL_dconic, dL_dcolor, dL_dxyz, dL_dscales,
                   (float4 *)dL_duquats, dL_dshs, cam, partials);
        else
            launch(preprocess_sh3_bwd_kernel<3>, gblocks, 256, 0, stream, P, xyz, scales, (const float4 *)uquats, intr,
                   extr, shs, depth, radius, (const float2 *)dL_duv, dL_dconic, dL_dcolor, dL_dxyz, dL_dscales,
                   (float4 *)dL_duquats, dL_dshs, cam, partials);
        if (cam) launch(cam_grad_finalize_kernel, 1, kCamGradFinalizeThreads, 0, stream, gblocks, partials,
                        dL_dintr, dL_dextr, 0);
        return check_launch("rasterize_preprocess_backward");
    }
    if (sh && D <= 16 && C <= kShChanBlock) {  // one kernel: SH and geometry adjoints
        const size_t smem = (size_t)256 * ((C * D) | 1) * sizeof(float);
#define MSPLAT_PREP_SH_BWD(DG)                                                                                   \
    case (DG + 1) * (DG + 1):                                                                                    \
        cudaFuncSetAttribute(preprocess_sh_bwd_kernel<DG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        launch(preprocess_sh_bwd_kernel<DG>, gblocks, 256, smem, stream, P, C, xyz, scales, (const float4 *)uquats, \
               intr, extr, shs, depth, radius, (const float2 *)dL_duv, dL_dconic, dL_dcolor, dL_dxyz, dL_dscales,  \
               (float4 *)dL_duquats, dL_dshs, cam, partials);                                                   \
        break;
        switch (D) {
            MSPLAT_PREP_SH_BWD(0) MSPLAT_PREP_SH_BWD(1) MSPLAT_PREP_SH_BWD(2) MSPLAT_PREP_SH_BWD(3)
            default: break;
        }
#undef MSPLAT_PREP_SH_BWD
        if (cam) launch(cam_grad_finalize_kernel, 1, kCamGradFinalizeThreads, 0, stream, gblocks, partials,
                        dL_dintr, dL_dextr, 0);
        return check_launch("rasterize_preprocess_backward");
    }
    if (sh) {
        // writes dL/dxyz (view-direction part) first; the geometry kernel adds
        const ShDirs in{nullptr, nullptr, xyz, extr, depth, dL_dxyz};
        const int st = sh_dispatch(true, P, C, D, shs, in, dL_dcolor, dL_dshs, nullptr, stream);
        if (st) return st;
    }
    launch(preprocess_bwd_kernel, gblocks, 256, 0, stream, P, xyz, scales, (const float4 *)uquats, intr, extr, depth,
           radius, (const float2 *)dL_duv, dL_dconic, sh, dL_dxyz, dL_dscales, (float4 *)dL_duquats, cam, partials);
    if (cam) launch(cam_grad_finalize_kernel, 1, kCamGradFinalizeThreads, 0, stream, gblocks, partials, dL_dintr,
                    dL_dextr, 0);
    return check_launch("rasterize_preprocess_backward");
}
