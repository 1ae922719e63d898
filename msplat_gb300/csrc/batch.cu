// Batched preprocess of one scene for B cameras (multi-camera rendering).
//
// No counterpart in the reference, which renders one camera per call
// (msplat/__init__.py:22-93).  The forward reads each Gaussian -- centre,
// scale, rotation and its SH coefficient rows -- once, computes its 3-D
// covariance once, and loops over the cameras, writing per-camera uv,
// depth, conic, radius, tiles and colour in camera-major [B, P, ...]
// layout, so every camera's slice feeds the single-camera sort and blend
// unchanged.  The per-camera arithmetic is the same device code as the
// single-camera fused path (geometry.cuh, sh_basis.cuh), so every camera's
// outputs are bit-identical to a single-camera call.
//
// The adjoint reads the per-camera blend gradients [B, P, ...] and sums the
// Gaussian's gradients over the cameras in registers (xyz, opacity, and
// dL/dcov, whose adjoint -- linear in it -- then gives the scale and
// rotation gradients once) and in a shared-memory row (SH coefficients), so each
// parameter gradient is written once instead of B times; camera gradients
// are reduced per warp and camera (a reduce-scatter of shuffles) into
// per-warp shared slots, which are summed in a fixed order into partial
// rows [B][blocks][16] once per kCamChunk cameras (two block barriers per
// chunk instead of two per camera).
#include "geometry.cuh"
#include "sh_basis.cuh"

namespace msplat {

constexpr int kCamChunk = 16;  // cameras per flush of the per-warp camera-gradient slots

// cams: [B][16] = intr (fx, fy, cx, cy) then extr (3x4 row-major);
// dims: [B][2] = (W, H).
__device__ __forceinline__ Cam load_batch_cam(const float *__restrict__ cams, int b) {
    return load_cam(cams + 16 * b, cams + 16 * b + 4);
}

// Same expressions as camera_centre / sh_direction<true> of the SH kernels.
__device__ __forceinline__ void view_direction(const float *__restrict__ extr, float px, float py, float pz,
                                               float (&d)[3], float &len) {
    float cc[3];
    camera_centre(extr, cc);
    const float dx = px - cc[0], dy = py - cc[1], dz = pz - cc[2];
    len = sqrtf(dx * dx + dy * dy + dz * dz);
    d[0] = dx / len;
    d[1] = dy / len;
    d[2] = dz / len;
}

template <int DEG>
__global__ void __launch_bounds__(256)
batch_preprocess_fwd_kernel(int P, int B, int C, const float *__restrict__ xyz, const float *__restrict__ scales,
                            const float4 *__restrict__ quats, const float *__restrict__ shs,
                            const float *__restrict__ cams, const int *__restrict__ dims, float nearest,
                            float extent, float2 *__restrict__ uv, float *__restrict__ depth,
                            float *__restrict__ conic, int32_t *__restrict__ radius, int32_t *__restrict__ tiles,
                            float *__restrict__ color) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    extern __shared__ float smem[];
    const int CD = C * D, stride = CD | 1;
    const int p0 = blockIdx.x * blockDim.x;
    const int n = min((int)blockDim.x, P - p0);
    if (C > 0) stage_rows(smem, shs + (size_t)p0 * CD, n, CD, stride);
    __syncthreads();
    const int t = threadIdx.x;
    if (t >= n) return;
    const int p = p0 + t;
    const float *row = smem + t * stride;
    const float px = xyz[3 * p], py = xyz[3 * p + 1], pz = xyz[3 * p + 2];
    float cov[6];
    cov3d_fwd_one(scales[3 * p], scales[3 * p + 1], scales[3 * p + 2], quats[p], cov);
    for (int b = 0; b < B; ++b) {
        const Cam c = load_batch_cam(cams, b);
        const int W = __ldg(dims + 2 * b), H = __ldg(dims + 2 * b + 1);
        const size_t q = (size_t)b * P + p;
        float2 u;
        float dep;
        project_fwd_one(c, px, py, pz, W, H, nearest, extent, u, dep);
        uv[q] = u;
        depth[q] = dep;
        float o[3] = {0.f, 0.f, 0.f};
        int rad = 0, nt = 0;
        if (dep != 0.0f) ewa_fwd_one(c, px, py, pz, cov, u, ceil_div(W, kTile), ceil_div(H, kTile), o, rad, nt);
        conic[3 * q + 0] = o[0];
        conic[3 * q + 1] = o[1];
        conic[3 * q + 2] = o[2];
        radius[q] = rad;
        tiles[q] = nt;
        if (C == 0) continue;
        float *out = color + q * C;
        if (dep == 0.0f) {
            for (int ch = 0; ch < C; ++ch) out[ch] = 0.f;
            continue;
        }
        float d[3], len;
        view_direction(cams + 16 * b + 4, px, py, pz, d, len);
        for (int c0 = 0; c0 < C; c0 += kShChanBlock) {
            float acc[kShChanBlock] = {0.f, 0.f, 0.f, 0.f};
            const int nc = min(kShChanBlock, C - c0);
            sh_basis<DEG, false>(d[0], d[1], d[2], [&](int i, float Y) {
#pragma unroll
                for (int cb = 0; cb < kShChanBlock; ++cb)
                    if (cb < nc) acc[cb] += Y * row[(c0 + cb) * D + i];
            });
            for (int cb = 0; cb < nc; ++cb) out[c0 + cb] = acc[cb];
        }
    }
}

// One camera's per-Gaussian inputs of the adjoint (zeros where the
// Gaussian is inactive or a pointer is null; the first 4 colour gradients).
struct BatchBwdIn {
    float depth;
    int radius;
    float2 duv;
    float dconic[3];
    float dcol[kShChanBlock];
    float dop;
};

__device__ __forceinline__ BatchBwdIn load_batch_bwd_in(bool active, size_t q, int C, const float *__restrict__ depth,
                                                        const int32_t *__restrict__ radius,
                                                        const float2 *__restrict__ dL_duv,
                                                        const float *__restrict__ dL_dconic,
                                                        const float *__restrict__ dL_dcolor,
                                                        const float *__restrict__ dL_dop_cam) {
    BatchBwdIn in;
    in.depth = active ? depth[q] : 0.0f;
    in.radius = active ? radius[q] : 0;
    in.duv = active ? dL_duv[q] : make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 3; ++k) in.dconic[k] = active ? dL_dconic[3 * q + k] : 0.f;
#pragma unroll
    for (int k = 0; k < kShChanBlock; ++k) in.dcol[k] = (active && k < C) ? dL_dcolor[q * C + k] : 0.f;
    in.dop = (active && dL_dop_cam) ? dL_dop_cam[q] : 0.f;
    return in;
}

// Shared memory per block: the coefficient rows, then (backward) one
// gradient-accumulator row per Gaussian.
// Up to degree 3 the adjoint fits 128 registers without spilling (4 blocks
// of 128 threads per SM); higher degrees keep the compiler's choice.
template <int DEG>
__global__ void __launch_bounds__(256, DEG <= 3 ? 2 : 1)
batch_preprocess_bwd_kernel(int P, int B, int C, const float *__restrict__ xyz, const float *__restrict__ scales,
                            const float4 *__restrict__ quats, const float *__restrict__ shs,
                            const float *__restrict__ cams, const float *__restrict__ depth,
                            const int32_t *__restrict__ radius, const float2 *__restrict__ dL_duv,
                            const float *__restrict__ dL_dconic, const float *__restrict__ dL_dcolor,
                            const float *__restrict__ dL_dop_cam, float *__restrict__ dL_dxyz,
                            float *__restrict__ dL_dscales, float4 *__restrict__ dL_dquats,
                            float *__restrict__ dL_dshs, float *__restrict__ dL_dopacity, bool cam_grads,
                            float *__restrict__ partials) {
    constexpr int D = (DEG + 1) * (DEG + 1);
    extern __shared__ float smem[];
    const int CD = C * D, stride = CD | 1;
    const int p0 = blockIdx.x * blockDim.x;
    const int n = min((int)blockDim.x, P - p0);
    const int nwarps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *grow_base = smem + (size_t)blockDim.x * stride;
    // per-warp camera-gradient slots [kCamChunk][warps][16] after the rows
    float *cslot = smem + (C > 0 ? (size_t)2 * blockDim.x * stride : 0);
    if (C > 0) {
        stage_rows(smem, shs + (size_t)p0 * CD, n, CD, stride);
        for (int e = threadIdx.x; e < n * stride; e += blockDim.x) grow_base[e] = 0.f;
    }
    __syncthreads();
    const int t = threadIdx.x;
    const bool active = t < n;
    const int p = active ? p0 + t : p0;
    const float *row = smem + t * stride;
    float *grow = grow_base + t * stride;
    float px = 0.f, py = 0.f, pz = 0.f, cov[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float s[3] = {0.f, 0.f, 0.f};
    float4 qt = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
        px = xyz[3 * p];
        py = xyz[3 * p + 1];
        pz = xyz[3 * p + 2];
        s[0] = scales[3 * p];
        s[1] = scales[3 * p + 1];
        s[2] = scales[3 * p + 2];
        qt = quats[p];
        cov3d_fwd_one(s[0], s[1], s[2], qt, cov);
    }
    // dL/dcov summed over the cameras: the covariance adjoint is linear in
    // it, so it runs once per Gaussian after the loop instead of per camera
    float gxyz[3] = {0.f, 0.f, 0.f}, gV[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, gop = 0.f;
    // The inputs of camera b + 1 are loaded while camera b is computed (the
    // loop is latency bound at this occupancy otherwise).
    BatchBwdIn cur = load_batch_bwd_in(active, (size_t)p, C, depth, radius, dL_duv, dL_dconic, dL_dcolor, dL_dop_cam);
    for (int b = 0; b < B; ++b) {
        const BatchBwdIn in = cur;
        if (b + 1 < B) cur = load_batch_bwd_in(active, (size_t)(b + 1) * P + p, C, depth, radius, dL_duv, dL_dconic,
                                                 dL_dcolor, dL_dop_cam);
        float acc[kCamGradVals];
#pragma unroll
        for (int k = 0; k < kCamGradVals; ++k) acc[k] = 0.f;
        const size_t q = (size_t)b * P + p;
        if (active && in.depth != 0.0f) {
            const Cam c = load_batch_cam(cams, b);
            float g[3] = {0.f, 0.f, 0.f};
            project_bwd_one(c, px, py, pz, in.duv, 0.0f, g, cam_grads, acc);
            if (in.radius > 0) {
                float ge[3], dV[6];
                if (ewa_bwd_one(c, px, py, pz, cov, in.dconic[0], in.dconic[1], in.dconic[2], ge, dV, cam_grads,
                                acc)) {
#pragma unroll
                    for (int k = 0; k < 6; ++k) gV[k] += dV[k];
#pragma unroll
                    for (int k = 0; k < 3; ++k) g[k] += ge[k];
                }
            }
            if (C > 0) {
                // SH adjoint on this camera's view direction: dL/dsh summed
                // over cameras in the shared row, the direction gradient
                // carried to v = x - c (dL/dx) and to the camera centre.
                float d[3], len;
                view_direction(cams + 16 * b + 4, px, py, pz, d, len);
                float gdx = 0.f, gdy = 0.f, gdz = 0.f;
                for (int c0 = 0; c0 < C; c0 += kShChanBlock) {
                    float gc[kShChanBlock] = {0.f, 0.f, 0.f, 0.f};
                    const int nc = min(kShChanBlock, C - c0);
                    if (c0 == 0) {
#pragma unroll
                        for (int cb = 0; cb < kShChanBlock; ++cb) gc[cb] = in.dcol[cb];
                    } else {
                        for (int cb = 0; cb < nc; ++cb) gc[cb] = dL_dcolor[q * C + c0 + cb];
                    }
                    sh_basis<DEG, true>(d[0], d[1], d[2], [&](int i, float Y, float yx, float yy, float yz) {
#pragma unroll
                        for (int cb = 0; cb < kShChanBlock; ++cb) {
                            if (cb < nc) {
                                const int k = (c0 + cb) * D + i;
                                const float w = gc[cb] * row[k];
                                gdx += w * yx;
                                gdy += w * yy;
                                gdz += w * yz;
                                grow[k] += gc[cb] * Y;
                            }
                        }
                    });
                }
                const float dg = d[0] * gdx + d[1] * gdy + d[2] * gdz;
                const float gv[3] = {(gdx - d[0] * dg) / len, (gdy - d[1] * dg) / len, (gdz - d[2] * dg) / len};
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
#pragma unroll
            for (int k = 0; k < 3; ++k) gxyz[k] += g[k];
        }
        gop += in.dop;
        if (cam_grads) {
            const int cb = b % kCamChunk;
            const float tot = warp_reduce_scatter_16(acc);
            if ((lane & 1) == 0) cslot[((size_t)cb * nwarps + warp) * kCamGradVals + (lane >> 1)] = tot;
            if (cb == kCamChunk - 1 || b == B - 1) {
                __syncthreads();
                // the block's partial row per camera of the chunk: its warps'
                // slots in warp order
                const int b0 = b - cb;
                for (int e = threadIdx.x; e < (cb + 1) * kCamGradVals; e += blockDim.x) {
                    const int c = e / kCamGradVals, k = e - c * kCamGradVals;
                    float s = 0.f;
                    for (int w = 0; w < nwarps; ++w) s += cslot[((size_t)c * nwarps + w) * kCamGradVals + k];
                    partials[((size_t)(b0 + c) * gridDim.x + blockIdx.x) * kCamGradVals + k] = s;
                }
                __syncthreads();  // the slots are reused by the next chunk
            }
        }
    }
    if (active) {
        float gs[3];
        float4 gq;
        cov3d_bwd_one(s, qt, gV, gs, gq);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            dL_dxyz[3 * p + k] = gxyz[k];
            dL_dscales[3 * p + k] = gs[k];
        }
        dL_dquats[p] = gq;
        if (dL_dopacity) dL_dopacity[p] = gop;
    }
    if (C > 0) {
        __syncthreads();
        unstage_rows(dL_dshs + (size_t)p0 * CD, grow_base, n, CD, stride);
    }
}

// Gaussians per block: the forward stages one row per Gaussian, the
// backward two; both stay under ~96 KB of shared memory.
// The longest coefficient rows (C * D floats) the batched backward stages:
// 32 Gaussians' rows and gradient rows and the camera-gradient slots in
// 200 KB of shared memory (the forward, rows alone, takes up to 1,599).
constexpr int kBatchMaxCD = 795;

inline int batch_block_points(int CD, bool backward) {
    const size_t row = (size_t)(CD | 1) * sizeof(float) * (backward ? 2 : 1);
    int nt = 256;
    while (nt > 32 && (size_t)nt * row > 96 * 1024) nt >>= 1;
    return nt;
}

}  // namespace msplat

using namespace msplat;

namespace {

int batch_degree(int C, int D) {
    if (C == 0) return 0;
    for (int l = 0; l <= kMaxShDeg; ++l)
        if ((l + 1) * (l + 1) == D) return l;
    return -1;
}

template <int DEG>
int batch_fwd_launch(int P, int B, int C, const float *xyz, const float *scales, const float *uquats,
                     const float *shs, const float *cams, const int *dims, float nearest, float extent, float *uv,
                     float *depth, float *conic, int32_t *radius, int32_t *tiles, float *color, cudaStream_t stream) {
    const int CD = C * (DEG + 1) * (DEG + 1);
    const int nt = batch_block_points(CD, false);
    const size_t smem = C > 0 ? (size_t)nt * (CD | 1) * sizeof(float) : 0;
    if (smem > 200 * 1024)
        return set_error(MSPLAT_ERR_UNSUPPORTED, "batch_preprocess_forward: C*D = %d too large (at most 1599)", CD);
    cudaFuncSetAttribute(batch_preprocess_fwd_kernel<DEG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    launch(batch_preprocess_fwd_kernel<DEG>, ceil_div(P, nt), nt, smem, stream, P, B, C, xyz, scales,
           (const float4 *)uquats, shs, cams, dims, nearest, extent, (float2 *)uv, depth, conic, radius, tiles, color);
    return check_launch("batch_preprocess_forward");
}

template <int DEG>
int batch_bwd_launch(int P, int B, int C, const float *xyz, const float *scales, const float *uquats,
                     const float *shs, const float *cams, const float *depth, const int32_t *radius,
                     const float *dL_duv, const float *dL_dconic, const float *dL_dcolor, const float *dL_dop_cam,
                     float *dL_dxyz, float *dL_dscales, float *dL_duquats, float *dL_dshs, float *dL_dopacity,
                     float *dL_dcams, float *partials, cudaStream_t stream) {
    const int CD = C * (DEG + 1) * (DEG + 1);
    const int nt = batch_block_points(CD, true);
    const int blocks = ceil_div(P, nt);
    const bool cam = dL_dcams != nullptr;
    const size_t smem = (C > 0 ? (size_t)2 * nt * (CD | 1) * sizeof(float) : 0) +
                        (cam ? (size_t)kCamChunk * (nt / 32) * kCamGradVals * sizeof(float) : 0);
    if (smem > 200 * 1024)
        return set_error(MSPLAT_ERR_UNSUPPORTED, "batch_preprocess_backward: C*D = %d too large (at most %d)", CD,
                         kBatchMaxCD);
    cudaFuncSetAttribute(batch_preprocess_bwd_kernel<DEG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    launch(batch_preprocess_bwd_kernel<DEG>, blocks, nt, smem, stream, P, B, C, xyz, scales, (const float4 *)uquats,
           shs, cams, depth, radius, (const float2 *)dL_duv, dL_dconic, dL_dcolor, dL_dop_cam, dL_dxyz, dL_dscales,
           (float4 *)dL_duquats, dL_dshs, dL_dopacity, cam, partials);
    // one finalize block per camera: rows [b][blocks][16] -> dL_dcams[b] =
    // (intr[4], extr[12])
    if (cam)
        launch(cam_grad_finalize_kernel, B, kCamGradFinalizeThreads, 0, stream, blocks, partials, dL_dcams,
               dL_dcams + 4, 16);
    return check_launch("batch_preprocess_backward");
}

}  // namespace

#define MSPLAT_BATCH_DEG_SWITCH(deg, CALL)                                                                      \
    switch (deg) {                                                                                              \
        case 0: return CALL(0); case 1: return CALL(1); case 2: return CALL(2); case 3: return CALL(3);          \
        case 4: return CALL(4); case 5: return CALL(5); case 6: return CALL(6); case 7: return CALL(7);          \
        case 8: return CALL(8); case 9: return CALL(9); case 10: return CALL(10);                                \
        default: return set_error(MSPLAT_ERR_UNSUPPORTED, "batch preprocess: D = %d is not (deg+1)^2", D);      \
    }

extern "C" size_t msplat_batch_preprocess_workspace_size(int P, int B, int C, int D) {
    if (P <= 0 || B <= 0) return 0;
    const int nt = batch_block_points(C * (C > 0 ? D : 0), true);
    return (size_t)B * ceil_div(P, nt) * kCamGradVals * sizeof(float);
}

extern "C" int msplat_batch_preprocess_forward(int P, int B, const float *xyz, const float *scales,
                                               const float *uquats, const float *cams, const int32_t *dims,
                                               float nearest, float extent, int C, int D, const float *shs,
                                               float *uv, float *depth, float *conic, int32_t *radius,
                                               int32_t *tiles, float *color, msplat_stream_t stream) {
    if (P < 0 || B < 0 || C < 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_preprocess_forward: bad sizes P=%d B=%d C=%d", P, B, C);
    if (P == 0 || B == 0) return MSPLAT_OK;
    if (!xyz || !scales || !uquats || !cams || !dims || !uv || !depth || !conic || !radius || !tiles ||
        (C > 0 && (!shs || !color)))
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_preprocess_forward: null pointer");
    if (((uintptr_t)uquats & 15) != 0 || ((uintptr_t)uv & 7) != 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_preprocess_forward: misaligned uquats / uv");
    if ((size_t)P * (size_t)B > (size_t)INT32_MAX * 4)
        return set_error(MSPLAT_ERR_CAPACITY, "batch_preprocess_forward: P * B too large");
    const int deg = batch_degree(C, D);
#define MSPLAT_CALL(L) \
    batch_fwd_launch<L>(P, B, C, xyz, scales, uquats, shs, cams, dims, nearest, extent, uv, depth, conic, radius, \
                        tiles, color, stream)
    MSPLAT_BATCH_DEG_SWITCH(deg, MSPLAT_CALL)
#undef MSPLAT_CALL
}

extern "C" int msplat_batch_preprocess_backward(int P, int B, const float *xyz, const float *scales,
                                                const float *uquats, const float *cams, int C, int D,
                                                const float *shs, const float *depth, const int32_t *radius,
                                                const float *dL_duv, const float *dL_dconic,
                                                const float *dL_dcolor, const float *dL_dopacity_cam,
                                                float *dL_dxyz, float *dL_dscales, float *dL_duquats,
                                                float *dL_dshs, float *dL_dopacity, float *dL_dcams,
                                                void *workspace, size_t workspace_bytes, msplat_stream_t stream) {
    if (P < 0 || B < 0 || C < 0) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_preprocess_backward: bad sizes");
    if (P == 0 || B == 0) {
        if (dL_dcams && B > 0) cudaMemsetAsync(dL_dcams, 0, (size_t)B * 16 * sizeof(float), stream);
        return check_launch("batch_preprocess_backward");
    }
    if (!xyz || !scales || !uquats || !cams || !depth || !radius || !dL_duv || !dL_dconic || !dL_dxyz ||
        !dL_dscales || !dL_duquats || (C > 0 && (!shs || !dL_dcolor || !dL_dshs)))
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_preprocess_backward: null pointer");
    if ((((uintptr_t)uquats | (uintptr_t)dL_duquats) & 15) != 0 || ((uintptr_t)dL_duv & 7) != 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_preprocess_backward: misaligned buffers");
    const size_t need = msplat_batch_preprocess_workspace_size(P, B, C, D);
    if (dL_dcams && (!workspace || workspace_bytes < need))
        return set_error(MSPLAT_ERR_WORKSPACE, "batch_preprocess_backward: workspace of %zu bytes < %zu",
                         workspace_bytes, need);
    const int deg = batch_degree(C, D);
#define MSPLAT_CALL(L)                                                                                         \
    batch_bwd_launch<L>(P, B, C, xyz, scales, uquats, shs, cams, depth, radius, dL_duv, dL_dconic, dL_dcolor,  \
                        dL_dopacity_cam, dL_dxyz, dL_dscales, dL_duquats, dL_dshs, dL_dopacity, dL_dcams,       \
                        (float *)workspace, stream)
    MSPLAT_BATCH_DEG_SWITCH(deg, MSPLAT_CALL)
#undef MSPLAT_CALL
}
