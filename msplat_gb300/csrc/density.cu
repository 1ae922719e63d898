// Density-control statistics: the step after the backward pass in
// training.  No kernel counterpart in the reference, whose training loop
// (tutorials/gs_3d.py:193-225) prunes and densifies on opacity and scale
// alone; its rasteriser exposes the screen-space gradient through `ndc`
// (msplat/alpha_blending.py:107-110), which is what this accumulates.
//
// Per Gaussian visible in the frame (radius > 0): grad_accum += |dL/dndc|
// (2-norm), count += 1, max_radius = max(max_radius, radius).  One thread
// per Gaussian, coalesced, HBM-bound (8 B read + 4 B radius + 12 B
// read-modify-write).
#include "common.cuh"

namespace msplat {

__global__ void __launch_bounds__(256)
density_stats_kernel(int P, const float2 *__restrict__ dL_dndc, const int32_t *__restrict__ radius,
                     float *__restrict__ grad_accum, int32_t *__restrict__ count, int32_t *__restrict__ max_radius) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int r = radius[i];
    if (r <= 0) return;
    const float2 g = dL_dndc[i];
    grad_accum[i] += sqrtf(g.x * g.x + g.y * g.y);
    count[i] += 1;
    max_radius[i] = max(max_radius[i], r);
}

}  // namespace msplat

using namespace msplat;

extern "C" int msplat_density_stats_update(int P, const float *dL_dndc, const int32_t *radius, float *grad_accum,
                                           int32_t *count, int32_t *max_radius, msplat_stream_t stream) {
    if (P < 0) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "density_stats_update: P < 0");
    if (P == 0) return MSPLAT_OK;
    if (!dL_dndc || !radius || !grad_accum || !count || !max_radius)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "density_stats_update: null pointer");
    if (((uintptr_t)dL_dndc & 7) != 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "density_stats_update: dL_dndc not 8-byte aligned");
    launch(density_stats_kernel, ceil_div(P, 256), 256, 0, stream, P, (const float2 *)dL_dndc, radius, grad_accum,
           count, max_radius);
    return check_launch("density_stats_update");
}
