// Internal interface of the SH kernels (compute_sh.cu) for the fused
// rasterisation (rasterize.cu).
#pragma once

#include "camgrad.cuh"
#include "sh_basis.cuh"

namespace msplat {

// Where a kernel takes its view directions: either a [P,3] array (with an
// optional visibility mask), or -- camera mode, used by the fused
// rasterisation -- from the Gaussian centres and the camera centre
// c = -R^T T of the extrinsics, d = (x - c) / |x - c|, with visibility
// depth != 0.  In camera mode the backward also carries dL/ddir back to the
// centres (written to dxyz); that value is also minus the gradient of the
// camera centre, which the caller folds into the extrinsics.
struct ShDirs {
    const float *dirs;
    const uint8_t *visible;
    const float *xyz;    // camera mode when non-null
    const float *extr;   // [3,4]
    const float *depth;  // [P]
    float *dxyz;         // backward, camera mode: [P,3] written
};

// Runs the SH forward (backward) for coefficients [P, C, D], D = (deg+1)^2,
// deg <= 10.  Backward: dL/dval -> dL/dshs (out) and, with `in.dirs`,
// dL/ddirs; in camera mode dL/dxyz goes to in.dxyz.
int sh_dispatch(bool backward, int P, int C, int D, const float *shs, const ShDirs &in, const float *dval,
                float *out, float *ddirs, cudaStream_t stream);

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

// The SH kernels for rows longer than a block's shared memory holds
// (compute_sh_sliced.cu): blocks of kShSlicedPoints Gaussians, their rows
// staged CC channels at a time into `smem` bytes.
constexpr int kShSlicedPoints = 32;
template <int DEG>
void sh_go_sliced(bool backward, int CC, size_t smem, int P, int C, const float *shs, const ShDirs &in,
                  const float *dval, float *out, float *ddirs, cudaStream_t stream);

}  // namespace msplat
