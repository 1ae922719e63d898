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
#include "geometry.cuh"

namespace msplat {

__global__ void __launch_bounds__(256)
ewa_fwd_kernel(int P, const float *__restrict__ xyz, const float *__restrict__ cov3d,
               const float *__restrict__ intr, const float *__restrict__ extr,
               const float2 *__restrict__ uv, int gx, int gy,
               const uint8_t *__restrict__ visible, float *__restrict__ conic,
               int32_t *__restrict__ radius, int32_t *__restrict__ tiles) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    float o[3] = {0.f, 0.f, 0.f};
    int rad = 0, nt = 0;
    if (!visible || visible[i]) {
        const Cam k = load_cam(intr, extr);
        ewa_fwd_one(k, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], cov3d + 6 * i, uv[i], gx, gy, o, rad, nt);
    }
    conic[3 * i + 0] = o[0];
    conic[3 * i + 1] = o[1];
    conic[3 * i + 2] = o[2];
    radius[i] = rad;
    tiles[i] = nt;
}

__global__ void __launch_bounds__(256)
ewa_bwd_kernel(int P, const float *__restrict__ xyz, const float *__restrict__ cov3d,
               const float *__restrict__ intr, const float *__restrict__ extr,
               const int32_t *__restrict__ radius, const float *__restrict__ dL_dconic,
               float *__restrict__ dL_dxyz, float *__restrict__ dL_dcov3d,
               bool cam_grads, float *__restrict__ partials) {
    const Cam k = load_cam(intr, extr);
    float acc[kCamGradVals];
#pragma unroll
    for (int q = 0; q < kCamGradVals; ++q) acc[q] = 0.0f;

    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        float dxyz[3] = {0.f, 0.f, 0.f};
        float dV[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (radius[i] > 0) {
            if (!ewa_bwd_one(k, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], cov3d + 6 * i, dL_dconic[3 * i],
                             dL_dconic[3 * i + 1], dL_dconic[3 * i + 2], dxyz, dV, cam_grads, acc)) {
#pragma unroll
                for (int q = 0; q < 3; ++q) dxyz[q] = 0.f;
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
    if (cam) launch(cam_grad_finalize_kernel, 1, kCamGradFinalizeThreads, 0, stream, blocks, partials, dL_dintr,
               dL_dextr, 0);
    return check_launch("ewa_project_backward");
}
