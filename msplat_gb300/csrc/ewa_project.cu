// EWA splatting of 3-D Gaussians to screen-space conics, forward/backward.
//
// Forward follows msplat/src/ewa_project.cu:16-83: J = d(uv)/d(t) of the
// pinhole map, T = J W (W = rotation of the extrinsics), cov2D = T V T^T
// plus a 0.3 px^2 dilation; det == 0 -> invisible; eigenvalue bound
// lambda = mid +- sqrt(max(0.1, mid^2 - det)); radius = ceil(3 sqrt(max
// lambda)); the 16x16 tile rectangle of (uv, radius); empty rectangle ->
// invisible; conic = inverse of cov2D.  The matrix products use the Mat3
// helper (glm's summation shape) and the divisions/square roots are the
// same source operations, compiled with the same fast-math flags as the
// reference, so radius and tiles_touched are bit-identical.
//
// Backward follows :85-252 (adjoint of the conic w.r.t. cov2D, of cov2D
// w.r.t. V and T, of T w.r.t. J and W, of J w.r.t. t, and of t w.r.t. xyz
// and the extrinsics), with the camera terms reduced per block rather than
// 25 contended float atomics per point.
#include "camgrad.cuh"
#include "mat3.cuh"

namespace msplat {

struct EwaCam {
    float e[12];
    float fx, fy;
};

__device__ __forceinline__ EwaCam load_ewa_cam(const float *intr, const float *extr) {
    EwaCam c;
#pragma unroll
    for (int k = 0; k < 12; ++k) c.e[k] = __ldg(extr + k);
    c.fx = __ldg(intr + 0);
    c.fy = __ldg(intr + 1);
    return c;
}

// Shared by forward and backward: camera-space centre, J, W, T and the
// dilated 2-D covariance (a, b, c) = (cov2D00 + 0.3, cov2D01, cov2D11 + 0.3).
struct EwaGeom {
    float tx, ty, tz;
    Mat3 J, Wm, T;
    float a, b, c;
};

__device__ __forceinline__ EwaGeom ewa_geometry(const EwaCam &k, float px, float py,
                                                float pz, const float *__restrict__ v) {
    EwaGeom g;
    g.tx = k.e[0] * px + k.e[1] * py + k.e[2] * pz + k.e[3];
    g.ty = k.e[4] * px + k.e[5] * py + k.e[6] * pz + k.e[7];
    g.tz = k.e[8] * px + k.e[9] * py + k.e[10] * pz + k.e[11];
    g.J = Mat3::cols(k.fx / g.tz, 0.0f, 0.0f,
                     0.0f, k.fy / g.tz, 0.0f,
                     -(k.fx * g.tx) / (g.tz * g.tz), -(k.fy * g.ty) / (g.tz * g.tz), 0.0f);
    g.Wm = Mat3::cols(k.e[0], k.e[4], k.e[8], k.e[1], k.e[5], k.e[9], k.e[2], k.e[6], k.e[10]);
    g.T = g.J * g.Wm;
    const Mat3 V = Mat3::cols(v[0], v[1], v[2], v[1], v[3], v[4], v[2], v[4], v[5]);
    const Mat3 cov2 = g.T * V * g.T.transposed();
    g.a = cov2.c[0][0] + 0.3f;
    g.b = cov2.c[0][1];
    g.c = cov2.c[1][1] + 0.3f;
    return g;
}

__global__ void __launch_bounds__(256)
ewa_fwd_kernel(int P, const float *__restrict__ xyz, const float *__restrict__ cov3d,
               const float *__restrict__ intr, const float *__restrict__ extr,
               const float2 *__restrict__ uv, int gx, int gy,
               const uint8_t *__restrict__ visible, float *__restrict__ conic,
               int32_t *__restrict__ radius, int32_t *__restrict__ tiles) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    float o0 = 0.f, o1 = 0.f, o2 = 0.f;
    int rad = 0, nt = 0;
    if (!visible || visible[i]) {
        const EwaCam k = load_ewa_cam(intr, extr);
        const EwaGeom g = ewa_geometry(k, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], cov3d + 6 * i);
        const float det = g.a * g.c - g.b * g.b;
        if (det != 0.0f) {
            const float mid = 0.5f * (g.a + g.c);
            const float l1 = mid + sqrtf(fmaxf(0.1f, mid * mid - det));
            const float l2 = mid - sqrtf(fmaxf(0.1f, mid * mid - det));
            const float r = ceilf(3.f * sqrtf(fmaxf(l1, l2)));
            const float2 p = uv[i];
            int x0, y0, x1, y1;
            tile_rect(p.x, p.y, (int)r, gx, gy, x0, y0, x1, y1);
            const int area = (x1 - x0) * (y1 - y0);
            if (area != 0) {
                const float inv_det = 1.f / det;
                o0 = g.c * inv_det;
                o1 = -g.b * inv_det;
                o2 = g.a * inv_det;
                rad = (int)r;
                nt = area;
            }
        }
    }
    conic[3 * i + 0] = o0;
    conic[3 * i + 1] = o1;
    conic[3 * i + 2] = o2;
    radius[i] = rad;
    tiles[i] = nt;
}

__global__ void __launch_bounds__(256)
ewa_bwd_kernel(int P, const float *__restrict__ xyz, const float *__restrict__ cov3d,
               const float *__restrict__ intr, const float *__restrict__ extr,
               const int32_t *__restrict__ radius, const float *__restrict__ dL_dconic,
               float *__restrict__ dL_dxyz, float *__restrict__ dL_dcov3d,
               bool cam_grads, float *__restrict__ partials) {
    const EwaCam k = load_ewa_cam(intr, extr);
    float acc[kCamGradVals];
#pragma unroll
    for (int q = 0; q < kCamGradVals; ++q) acc[q] = 0.0f;

    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        float dxyz[3] = {0.f, 0.f, 0.f};
        float dV[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const float px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
        const float *v = cov3d + 6 * i;
        bool active = radius[i] > 0;
        EwaGeom g;
        float det = 0.f;
        if (active) {
            g = ewa_geometry(k, px, py, pz, v);
            det = g.a * g.c - g.b * g.b;
            active = det != 0.0f;
        }
        if (active) {
            const float gc0 = dL_dconic[3 * i], gc1 = dL_dconic[3 * i + 1], gc2 = dL_dconic[3 * i + 2];
            // conic = (c, -b, a) / det with det = a c - b^2.
            const float inv2 = 1.0f / (det * det);
            const float da = inv2 * (-g.c * g.c * gc0 + g.b * g.c * gc1 + (det - g.a * g.c) * gc2);
            const float db = inv2 * (2.f * g.b * g.c * gc0 - (det + 2.f * g.b * g.b) * gc1 +
                                     2.f * g.a * g.b * gc2);
            const float dc = inv2 * ((det - g.a * g.c) * gc0 + g.a * g.b * gc1 - g.a * g.a * gc2);
            // Rows 0 and 1 of T in maths order: T0[k] = T(0,k), T1[k] = T(1,k).
            float T0[3], T1[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) { T0[q] = g.T.c[q][0]; T1[q] = g.T.c[q][1]; }
            const float Vm[3][3] = {{v[0], v[1], v[2]}, {v[1], v[3], v[4]}, {v[2], v[4], v[5]}};
            // cov2D(0,0) = T0 V T0, cov2D(0,1) = T0 V T1, cov2D(1,1) = T1 V T1.
            dV[0] = T0[0] * T0[0] * da + T0[0] * T1[0] * db + T1[0] * T1[0] * dc;
            dV[3] = T0[1] * T0[1] * da + T0[1] * T1[1] * db + T1[1] * T1[1] * dc;
            dV[5] = T0[2] * T0[2] * da + T0[2] * T1[2] * db + T1[2] * T1[2] * dc;
            dV[1] = 2.f * T0[0] * T0[1] * da + (T0[0] * T1[1] + T0[1] * T1[0]) * db + 2.f * T1[0] * T1[1] * dc;
            dV[2] = 2.f * T0[0] * T0[2] * da + (T0[0] * T1[2] + T0[2] * T1[0]) * db + 2.f * T1[0] * T1[2] * dc;
            dV[4] = 2.f * T0[1] * T0[2] * da + (T0[1] * T1[2] + T0[2] * T1[1]) * db + 2.f * T1[1] * T1[2] * dc;
            float VT0[3], VT1[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                VT0[q] = Vm[q][0] * T0[0] + Vm[q][1] * T0[1] + Vm[q][2] * T0[2];
                VT1[q] = Vm[q][0] * T1[0] + Vm[q][1] * T1[1] + Vm[q][2] * T1[2];
            }
            float dT0[3], dT1[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                dT0[q] = 2.f * VT0[q] * da + VT1[q] * db;
                dT1[q] = VT0[q] * db + 2.f * VT1[q] * dc;
            }
            // T = J R: T(0,:) = J00 R0 + J02 R2, T(1,:) = J11 R1 + J12 R2.
            const float *R0 = k.e, *R1 = k.e + 4, *R2 = k.e + 8;
            const float dJ00 = R0[0] * dT0[0] + R0[1] * dT0[1] + R0[2] * dT0[2];
            const float dJ02 = R2[0] * dT0[0] + R2[1] * dT0[1] + R2[2] * dT0[2];
            const float dJ11 = R1[0] * dT1[0] + R1[1] * dT1[1] + R1[2] * dT1[2];
            const float dJ12 = R2[0] * dT1[0] + R2[1] * dT1[1] + R2[2] * dT1[2];
            const float iz = 1.f / g.tz, iz2 = iz * iz, iz3 = iz2 * iz;
            const float dtx = -k.fx * iz2 * dJ02;
            const float dty = -k.fy * iz2 * dJ12;
            const float dtz = -k.fx * iz2 * dJ00 - k.fy * iz2 * dJ11 +
                              2.f * k.fx * g.tx * iz3 * dJ02 + 2.f * k.fy * g.ty * iz3 * dJ12;
            dxyz[0] = R0[0] * dtx + R1[0] * dty + R2[0] * dtz;
            dxyz[1] = R0[1] * dtx + R1[1] * dty + R2[1] * dtz;
            dxyz[2] = R0[2] * dtx + R1[2] * dty + R2[2] * dtz;
            if (cam_grads) {
                const float J00 = g.J.c[0][0], J11 = g.J.c[1][1];
                const float J02 = g.J.c[2][0], J12 = g.J.c[2][1];
                acc[0] += iz * dJ00 - g.tx * iz2 * dJ02;
                acc[1] += iz * dJ11 - g.ty * iz2 * dJ12;
                const float pt[3] = {px, py, pz};
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    // Through T = J R ...
                    acc[4 + q] += J00 * dT0[q];
                    acc[8 + q] += J11 * dT1[q];
                    acc[12 + q] += J02 * dT0[q] + J12 * dT1[q];
                    // ... and through t = R x + T.
                    acc[4 + q] += pt[q] * dtx;
                    acc[8 + q] += pt[q] * dty;
                    acc[12 + q] += pt[q] * dtz;
                }
                acc[7] += dtx;
                acc[11] += dty;
                acc[15] += dtz;
            }
        }
        dL_dxyz[3 * i + 0] = dxyz[0];
        dL_dxyz[3 * i + 1] = dxyz[1];
        dL_dxyz[3 * i + 2] = dxyz[2];
#pragma unroll
        for (int q = 0; q < 6; ++q) dL_dcov3d[6 * i + q] = dV[q];
    }
    if (cam_grads) block_partial_16(acc, partials);
}

}  // namespace msplat

using namespace msplat;

extern "C" int msplat_ewa_project_forward(int P, const float *xyz, const float *cov3d,
                                          const float *intr, const float *extr,
                                          const float *uv, int W, int H,
                                          const uint8_t *visible, float *conic,
                                          int32_t *radius, int32_t *tiles,
                                          msplat_stream_t stream) {
    if (P < 0 || W <= 0 || H <= 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "ewa_project_forward: bad sizes P=%d W=%d H=%d", P, W, H);
    if (P == 0) return MSPLAT_OK;
    if (!xyz || !cov3d || !intr || !extr || !uv || !conic || !radius || !tiles)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "ewa_project_forward: null pointer");
    const int gx = ceil_div(W, kTile), gy = ceil_div(H, kTile);
    launch(ewa_fwd_kernel, ceil_div(P, 256), 256, 0, stream, P, xyz, cov3d, intr, extr, (const float2 *)uv,
                                                         gx, gy, visible, conic, radius, tiles);
    return check_launch("ewa_project_forward");
}

extern "C" int msplat_ewa_project_backward(int P, const float *xyz, const float *cov3d,
                                           const float *intr, const float *extr,
                                           const int32_t *radius, const float *dL_dconic,
                                           float *dL_dxyz, float *dL_dcov3d, float *dL_dintr,
                                           float *dL_dextr, void *workspace,
                                           size_t workspace_bytes, msplat_stream_t stream) {
    if (P < 0) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "ewa_project_backward: P < 0");
    const bool cam = dL_dintr || dL_dextr;
    if (P == 0) {
        if (dL_dintr) cudaMemsetAsync(dL_dintr, 0, 4 * sizeof(float), stream);
        if (dL_dextr) cudaMemsetAsync(dL_dextr, 0, 12 * sizeof(float), stream);
        return check_launch("ewa_project_backward");
    }
    if (!xyz || !cov3d || !intr || !extr || !radius || !dL_dconic || !dL_dxyz || !dL_dcov3d)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "ewa_project_backward: null pointer");
    if (cam && (!workspace || workspace_bytes < cam_grad_workspace_bytes()))
        return set_error(MSPLAT_ERR_WORKSPACE, "ewa_project_backward: workspace of %zu bytes < %zu",
                         workspace_bytes, cam_grad_workspace_bytes());
    const int blocks = min(ceil_div(P, 256), kCamGradBlocks);
    float *partials = (float *)workspace;
    launch(ewa_bwd_kernel, blocks, 256, 0, stream, P, xyz, cov3d, intr, extr, radius, dL_dconic,
                                               dL_dxyz, dL_dcov3d, cam, partials);
    if (cam) launch(cam_grad_finalize_kernel, 1, 32 * kCamGradVals, 0, stream, blocks, partials, dL_dintr, dL_dextr);
    return check_launch("ewa_project_backward");
}
