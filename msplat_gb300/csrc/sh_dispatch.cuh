// Internal interface of the SH kernels (compute_sh.cu) for the fused
// rasterisation (rasterize.cu).
#pragma once

#include "camgrad.cuh"

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

}  // namespace msplat
