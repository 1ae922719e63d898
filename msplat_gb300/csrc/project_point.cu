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
#include "camgrad.cuh"

namespace msplat {

struct Cam {
    float e[12];
    float fx, fy, cx, cy;
};

__device__ __forceinline__ Cam load_cam(const float *intr, const float *extr) {
    Cam c;
#pragma unroll
    for (int k = 0; k < 12; ++k) c.e[k] = __ldg(extr + k);
    c.fx = __ldg(intr + 0);
    c.fy = __ldg(intr + 1);
    c.cx = __ldg(intr + 2);
    c.cy = __ldg(intr + 3);
    return c;
}

__global__ void __launch_bounds__(256)
project_point_fwd_kernel(int P, const float *__restrict__ xyz,
                         const float *__restrict__ intr,
                         const float *__restrict__ extr, int W, int H,
                         float nearest, float extent, float2 *__restrict__ uv,
                         float *__restrict__ depth) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const Cam c = load_cam(intr, extr);
    const float px = xyz[3 * i + 0], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];

    // Same expression shape as the reference so the compiler contracts the
    // same products into FMAs.
    const float tx = c.e[0] * px + c.e[1] * py + c.e[2] * pz + c.e[3];
    const float ty = c.e[4] * px + c.e[5] * py + c.e[6] * pz + c.e[7];
    const float tz = c.e[8] * px + c.e[9] * py + c.e[10] * pz + c.e[11];
    const float inv_z = (float)(1.0 / ((double)tz + 1e-7));
    const float u = (float)((double)(c.fx * tx * inv_z + c.cx) - 0.5);
    const float v = (float)((double)(c.fy * ty * inv_z + c.cy) - 0.5);

    bool culled = (nearest > 0.0f) && (tz <= nearest);
    if (extent > 0.0f) {
        // (1 - extent) * W in float, then * 0.5 in double, as the reference.
        const float xlo = (float)((double)((1.0f - extent) * (float)W) * 0.5);
        const float xhi = (float)((double)((1.0f + extent) * (float)W) * 0.5);
        const float ylo = (float)((double)((1.0f - extent) * (float)H) * 0.5);
        const float yhi = (float)((double)((1.0f + extent) * (float)H) * 0.5);
        culled |= (u < xlo) || (u > xhi) || (v < ylo) || (v > yhi);
    }
    uv[i] = culled ? make_float2(0.0f, 0.0f) : make_float2(u, v);
    depth[i] = culled ? 0.0f : tz;
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
        const float px = xyz[3 * i + 0], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
        float gx = 0.0f, gy = 0.0f, gz = 0.0f;
        if (depth[i] != 0.0f) {  // depth == 0 marks a culled point
            const float tx = c.e[0] * px + c.e[1] * py + c.e[2] * pz + c.e[3];
            const float ty = c.e[4] * px + c.e[5] * py + c.e[6] * pz + c.e[7];
            const float tz = c.e[8] * px + c.e[9] * py + c.e[10] * pz + c.e[11];
            const float iz = (float)(1.0 / (double)tz);
            const float iz2 = (float)(1.0 / (double)(tz * tz));
            const float2 g = dL_duv[i];
            const float gd = dL_ddepth[i];
            // dL/dt for t = R x + T.
            const float dtx = c.fx * iz * g.x;
            const float dty = c.fy * iz * g.y;
            const float dtz = -(c.fx * tx * g.x + c.fy * ty * g.y) * iz2 + gd;
            gx = c.e[0] * dtx + c.e[4] * dty + c.e[8] * dtz;
            gy = c.e[1] * dtx + c.e[5] * dty + c.e[9] * dtz;
            gz = c.e[2] * dtx + c.e[6] * dty + c.e[10] * dtz;
            if (cam_grads) {
                acc[0] += tx * iz * g.x;
                acc[1] += ty * iz * g.y;
                acc[2] += g.x;
                acc[3] += g.y;
                const float pt[4] = {px, py, pz, 1.0f};
                const float dt[3] = {dtx, dty, dtz};
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc[4 + 4 * r + q] += dt[r] * pt[q];
            }
        }
        dL_dxyz[3 * i + 0] = gx;
        dL_dxyz[3 * i + 1] = gy;
        dL_dxyz[3 * i + 2] = gz;
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
        launch(cam_grad_finalize_kernel, 1, 32 * kCamGradVals, 0, stream, blocks, partials, dL_dintr, dL_dextr);
    return check_launch("project_point_backward");
}
