// Pinhole projection of Gaussian centres, forward and backward.
//
// Forward follows msplat/src/project_point.cu:13-57: t = R x + T,
// uv = (fx tx / tz + cx - 0.5, fy ty / tz + cy - 0.5), depth = tz, with the
// same mixed float/double arithmetic (1/(tz + 1e-7) and the -0.5 are double
// in the reference) so uv and depth are bit-identical.  Culled points are 0.
//
// Backward follows msplat/src/project_point.cu:59-145 for dL/dxyz and the
// camera gradients, but reduces the camera terms per block (warp shuffles,
// then a fixed-order pass over block partials) instead of issuing 20 global
// atomics per point onto 16 addresses.
#include "geometry.cuh"

namespace msplat {

__global__ void __launch_bounds__(256)
project_point_fwd_kernel(int P, const float *__restrict__ xyz,
                         const float *__restrict__ intr,
                         const float *__restrict__ extr, int W, int H,
                         float nearest, float extent, float2 *__restrict__ uv,
                         float *__restrict__ depth) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const Cam c = load_cam(intr, extr);
    float2 u;
    float d;
    project_fwd_one(c, xyz[3 * i + 0], xyz[3 * i + 1], xyz[3 * i + 2], W, H, nearest, extent, u, d);
    uv[i] = u;
    depth[i] = d;
}

__global__ void __launch_bounds__(256)
project_point_bwd_kernel(int P, const float *__restrict__ xyz,
                         const float *__restrict__ intr,
                         const float *__restrict__ extr,
                         const float *__restrict__ depth,
                         const float2 *__restrict__ dL_duv,
                         const float *__restrict__ dL_ddepth,
                         float *__restrict__ dL_dxyz, bool cam_grads,
                         float *__restrict__ partials) {
    const Cam c = load_cam(intr, extr);
    float acc[kCamGradVals];
#pragma unroll
    for (int k = 0; k < kCamGradVals; ++k) acc[k] = 0.0f;

    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P;
         i += gridDim.x * blockDim.x) {
        float g[3] = {0.0f, 0.0f, 0.0f};
        if (depth[i] != 0.0f)  // depth == 0 marks a culled point
            project_bwd_one(c, xyz[3 * i + 0], xyz[3 * i + 1], xyz[3 * i + 2], dL_duv[i], dL_ddepth[i], g,
                            cam_grads, acc);
        dL_dxyz[3 * i + 0] = g[0];
        dL_dxyz[3 * i + 1] = g[1];
        dL_dxyz[3 * i + 2] = g[2];
    }
    if (cam_grads) block_partial_16(acc, partials);
}

}  // namespace msplat

using namespace msplat;

extern "C" int msplat_project_point_forward(int P, const float *xyz,
                                            const float *intr,
                                            const float *extr, int W, int H,
                                            float nearest, float extent,
                                            float *uv, float *depth,
                                            msplat_stream_t stream) {
    if (P < 0 || W <= 0 || H <= 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT,
                         "project_point_forward: bad sizes P=%d W=%d H=%d", P, W, H);
    if (P == 0) return MSPLAT_OK;
    if (!xyz || !intr || !extr || !uv || !depth)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "project_point_forward: null pointer");
    launch(project_point_fwd_kernel, ceil_div(P, 256), 256, 0, stream,
        P, xyz, intr, extr, W, H, nearest, extent, (float2 *)uv, depth);
    return check_launch("project_point_forward");
}

extern "C" size_t msplat_camera_grad_workspace_size(int P) {
    (void)P;
    return cam_grad_workspace_bytes();
}

extern "C" int msplat_project_point_backward(
    int P, const float *xyz, const float *intr, const float *extr, int W,
    int H, const float *uv, const float *depth, const float *dL_duv,
    const float *dL_ddepth, float *dL_dxyz, float *dL_dintr, float *dL_dextr,
    void *workspace, size_t workspace_bytes, msplat_stream_t stream) {
    (void)W; (void)H; (void)uv;
    if (P < 0) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "project_point_backward: P < 0");
    const bool cam = dL_dintr || dL_dextr;
    if (P == 0) {
        if (cam) {
            if (dL_dintr) cudaMemsetAsync(dL_dintr, 0, 4 * sizeof(float), stream);
            if (dL_dextr) cudaMemsetAsync(dL_dextr, 0, 12 * sizeof(float), stream);
        }
        return check_launch("project_point_backward");
    }
    if (!xyz || !intr || !extr || !depth || !dL_duv || !dL_ddepth || !dL_dxyz)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "project_point_backward: null pointer");
    const int blocks = min(ceil_div(P, 256), kCamGradBlocks);
    if (cam && (!workspace || workspace_bytes < msplat_camera_grad_workspace_size(P)))
        return set_error(MSPLAT_ERR_WORKSPACE, "project_point_backward: workspace of %zu bytes < %zu",
                         workspace_bytes, msplat_camera_grad_workspace_size(P));
    float *partials = (float *)workspace;
    launch(project_point_bwd_kernel, blocks, 256, 0, stream,
        P, xyz, intr, extr, depth, (const float2 *)dL_duv, dL_ddepth, dL_dxyz, cam, partials);
    if (cam)
        launch(cam_grad_finalize_kernel, 1, kCamGradFinalizeThreads, 0, stream, blocks, partials, dL_dintr,
               dL_dextr, 0);
    return check_launch("project_point_backward");
}
