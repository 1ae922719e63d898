// 3-D covariance from scale and unit quaternion, forward and backward.
//
// Forward follows msplat/src/compute_cov3d.cu:24-58: with R the glm-style
// column-major rotation built from q = (r, x, y, z) and S = diag(scale),
// M = S * R and Sigma = M^T * M, stored as its upper triangle
// [s00, s01, s02, s11, s12, s22].  The Mat3 helper keeps glm's summation
// shape so Sigma is bit-identical.  Backward follows :60-117 (no
// normalisation adjoint: the quaternion is taken as already unit length).
// Points with visible == 0 produce zeros.
#include "common.cuh"
#include "mat3.cuh"

namespace msplat {

__device__ __forceinline__ Mat3 quat_to_rot_cols(float r, float x, float y, float z) {
    return Mat3::cols(1.f - 2.f * (y * y + z * z), 2.f * (x * y - r * z), 2.f * (x * z + r * y),
                      2.f * (x * y + r * z), 1.f - 2.f * (x * x + z * z), 2.f * (y * z - r * x),
                      2.f * (x * z - r * y), 2.f * (y * z + r * x), 1.f - 2.f * (x * x + y * y));
}

__device__ __forceinline__ Mat3 diag_scale(float sx, float sy, float sz) {
    return Mat3::cols(sx, 0.f, 0.f, 0.f, sy, 0.f, 0.f, 0.f, sz);
}

__global__ void __launch_bounds__(256)
cov3d_fwd_kernel(int P, const float *__restrict__ scales,
                 const float4 *__restrict__ quats, const uint8_t *__restrict__ visible,
                 float *__restrict__ cov3d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    float out[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (!visible || visible[i]) {
        const float4 q = quats[i];
        const Mat3 S = diag_scale(scales[3 * i], scales[3 * i + 1], scales[3 * i + 2]);
        const Mat3 R = quat_to_rot_cols(q.x, q.y, q.z, q.w);
        const Mat3 M = S * R;
        const Mat3 Sig = M.transposed() * M;
        out[0] = Sig.c[0][0];
        out[1] = Sig.c[0][1];
        out[2] = Sig.c[0][2];
        out[3] = Sig.c[1][1];
        out[4] = Sig.c[1][2];
        out[5] = Sig.c[2][2];
    }
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
        const float4 q = quats[i];
        const float r = q.x, x = q.y, y = q.z, z = q.w;
        const float s[3] = {scales[3 * i], scales[3 * i + 1], scales[3 * i + 2]};
        // Standard rotation Rs(i,j); the glm matrix of the forward is its
        // transpose, so M(i,j) = s_i * Rs(j,i) and Sigma = Rs S^2 Rs^T.
        float Rs[3][3];
        Rs[0][0] = 1.f - 2.f * (y * y + z * z); Rs[0][1] = 2.f * (x * y - r * z); Rs[0][2] = 2.f * (x * z + r * y);
        Rs[1][0] = 2.f * (x * y + r * z); Rs[1][1] = 1.f - 2.f * (x * x + z * z); Rs[1][2] = 2.f * (y * z - r * x);
        Rs[2][0] = 2.f * (x * z - r * y); Rs[2][1] = 2.f * (y * z + r * x); Rs[2][2] = 1.f - 2.f * (x * x + y * y);
        const float *g = dL_dcov + 6 * i;
        // Symmetric dL/dSigma: off-diagonal entries of the 6-vector stand for
        // both (i,j) and (j,i).
        const float G[3][3] = {{g[0], 0.5f * g[1], 0.5f * g[2]},
                               {0.5f * g[1], g[3], 0.5f * g[4]},
                               {0.5f * g[2], 0.5f * g[4], g[5]}};
        // Sigma = A A^T with A = Rs S: dL/dA = 2 G A.
        float A[3][3], dA[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) A[a][b] = Rs[a][b] * s[b];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
                dA[a][b] = 2.f * (G[a][0] * A[0][b] + G[a][1] * A[1][b] + G[a][2] * A[2][b]);
        // A(a,b) = Rs(a,b) s_b.
        float Gr[3][3];
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            ds[b] = dA[0][b] * Rs[0][b] + dA[1][b] * Rs[1][b] + dA[2][b] * Rs[2][b];
#pragma unroll
            for (int a = 0; a < 3; ++a) Gr[a][b] = dA[a][b] * s[b];
        }
        // Quaternion adjoint of the standard rotation matrix.
        dq.x = 2.f * z * (Gr[1][0] - Gr[0][1]) + 2.f * y * (Gr[0][2] - Gr[2][0]) +
               2.f * x * (Gr[2][1] - Gr[1][2]);
        dq.y = 2.f * y * (Gr[0][1] + Gr[1][0]) + 2.f * z * (Gr[0][2] + Gr[2][0]) +
               2.f * r * (Gr[2][1] - Gr[1][2]) - 4.f * x * (Gr[1][1] + Gr[2][2]);
        dq.z = 2.f * x * (Gr[0][1] + Gr[1][0]) + 2.f * r * (Gr[0][2] - Gr[2][0]) +
               2.f * z * (Gr[1][2] + Gr[2][1]) - 4.f * y * (Gr[0][0] + Gr[2][2]);
        dq.w = 2.f * r * (Gr[1][0] - Gr[0][1]) + 2.f * x * (Gr[0][2] + Gr[2][0]) +
               2.f * y * (Gr[1][2] + Gr[2][1]) - 4.f * z * (Gr[0][0] + Gr[1][1]);
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
