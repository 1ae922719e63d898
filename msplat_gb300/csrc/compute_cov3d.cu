// 3-D covariance from scale and unit quaternion, forward and backward.
//
// Forward follows msplat/src/compute_cov3d.cu:24-58: with R the glm-style
// column-major rotation built from q = (r, x, y, z) and S = diag(scale),
// M = S * R and Sigma = M^T * M, stored as its upper triangle
// [s00, s01, s02, s11, s12, s22].  The Mat3 helper keeps glm's summation
// shape so Sigma is bit-identical.  Backward follows :60-117 (no
// normalisation adjoint: the quaternion is taken as already unit length).
// Points with visible == 0 produce zeros.
#include "geometry.cuh"

namespace msplat {

__global__ void __launch_bounds__(256)
cov3d_fwd_kernel(int P, const float *__restrict__ scales,
                 const float4 *__restrict__ quats, const uint8_t *__restrict__ visible,
                 float *__restrict__ cov3d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    float out[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (!visible || visible[i]) cov3d_fwd_one(scales[3 * i], scales[3 * i + 1], scales[3 * i + 2], quats[i], out);
#pragma unroll
    for (int k = 0; k < 6; ++k) cov3d[6 * i + k] = out[k];
}

__global__ void __launch_bounds__(256)
cov3d_bwd_kernel(int P, const float *__restrict__ scales,
                 const float4 *__restrict__ quats, const uint8_t *__restrict__ visible,
                 const float *__restrict__ dL_dcov, float *__restrict__ dL_dscales,
                 float4 *__restrict__ dL_dquats) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    float ds[3] = {0.f, 0.f, 0.f};
    float4 dq = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!visible || visible[i]) {
        const float s[3] = {scales[3 * i], scales[3 * i + 1], scales[3 * i + 2]};
        cov3d_bwd_one(s, quats[i], dL_dcov + 6 * i, ds, dq);
    }
    dL_dscales[3 * i + 0] = ds[0];
    dL_dscales[3 * i + 1] = ds[1];
    dL_dscales[3 * i + 2] = ds[2];
    dL_dquats[i] = dq;
}

}  // namespace msplat

using namespace msplat;

extern "C" int msplat_compute_cov3d_forward(int P, const float *scales,
                                            const float *uquats,
                                            const uint8_t *visible, float *cov3d,
                                            msplat_stream_t stream) {
    if (P < 0) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_cov3d_forward: P < 0");
    if (P == 0) return MSPLAT_OK;
    if (!scales || !uquats || !cov3d)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_cov3d_forward: null pointer");
    if (((uintptr_t)uquats & 15) != 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_cov3d_forward: uquats not 16-byte aligned");
    launch(cov3d_fwd_kernel, ceil_div(P, 256), 256, 0, stream, P, scales, (const float4 *)uquats,
                                                           visible, cov3d);
    return check_launch("compute_cov3d_forward");
}

extern "C" int msplat_compute_cov3d_backward(int P, const float *scales,
                                             const float *uquats,
                                             const uint8_t *visible,
                                             const float *dL_dcov3d,
                                             float *dL_dscales, float *dL_duquats,
                                             msplat_stream_t stream) {
    if (P < 0) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_cov3d_backward: P < 0");
    if (P == 0) return MSPLAT_OK;
    if (!scales || !uquats || !dL_dcov3d || !dL_dscales || !dL_duquats)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_cov3d_backward: null pointer");
    if ((((uintptr_t)uquats | (uintptr_t)dL_duquats) & 15) != 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_cov3d_backward: quaternion buffers not 16-byte aligned");
    launch(cov3d_bwd_kernel, ceil_div(P, 256), 256, 0, stream, P, scales, (const float4 *)uquats, visible,
                                                           dL_dcov3d, dL_dscales, (float4 *)dL_duquats);
    return check_launch("compute_cov3d_backward");
}
