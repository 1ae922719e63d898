// Tile-based front-to-back alpha blending of depth-sorted 2-D Gaussians.
//
// Semantics follow msplat/src/alpha_blending.cu (forward :16-110, backward
// :112-246): one 16x16 tile per CTA, pixel centres at integer coordinates,
//   power = -0.5 (a dx^2 + c dy^2) - b dx dy        (skip if > 0)
//   alpha = min(0.99, opacity * exp(power))          (skip if < 1/255)
//   stop before a Gaussian that would take T below 1e-4,
//   out = sum f alpha T + T bg, ncontrib = list index of the last blended.
// The per-pair arithmetic is written as in the reference so T, ncontrib and
// the colours agree to the last bit where the exponential does.
//
// What is different (results unchanged):
//  * each batch of the tile's list is gathered once into shared memory
//    (geometry and features), and Gaussians whose alpha >= 1/255 ellipse
//    misses the whole tile are dropped there by a conservative box test;
//    survivors keep their list index so ncontrib counts every entry;
//  * per pair, exp is skipped when power is below a per-Gaussian bound that
//    already implies alpha < 1/255;
//  * any channel count runs in one pass up to 32 channels (the reference
//    re-runs the whole blend per chunk of <= 32 and transposes features);
//  * backward starts at the tile's largest ncontrib instead of the end of
//    the list, and per-Gaussian gradients are summed over each warp with a
//    reduce-scatter of shuffles before one atomic per value per warp (the
//    reference issues C + 6 atomics per pixel-Gaussian pair);
//  * in the C <= 4 kernels each warp owns an 8-column block of the tile and
//    walks only the gathered Gaussians whose alpha >= 1/255 ellipse reaches
//    that block (a conservative per-Gaussian mask built in the gather).
#include "batch_plan.cuh"
#include "cull.cuh"

namespace msplat {

// A multi-camera batch (batch_plan.cuh): one grid over every camera's
// tiles.  Per block, the camera of its tile gives the image size and the
// offsets into the stacked per-camera arrays; features are stacked per
// camera (feat_per_cam, rows like uv) or per scene (rows like opacity).
struct BlendBatch {
    BatchPlanView pv;
    int feat_per_cam;
};

// Where a block renders: its tile (coordinates, row of tile_range, split
// part), the image size, and in a multi-camera batch (BATCH) the offsets of
// the tile's camera into the stacked arrays (zero for a single camera).
struct BlendSite {
    int tx, ty, tidx, part, W, H, P;  // P: the Gaussians (rows) list ids index
    int64_t row_off, op_off, feat_off, pix_off;
};

template <bool BATCH, int SPLIT>
__device__ __forceinline__ BlendSite blend_site(const BlendBatch &bb, int P, int W, int H) {
    BlendSite s;
    if (BATCH) {
        const int t = blockIdx.x;
        const int b = batch_camera_of_tile(bb.pv, t);
        const BatchCam &c = bb.pv.cams[b];
        s.W = c.W;
        s.H = c.H;
        s.P = c.P;
        const int lt = t - c.tile_off;
        s.ty = lt / c.gx;
        s.tx = lt - s.ty * c.gx;
        s.tidx = t;
        s.part = 0;
        s.row_off = c.row_off;
        s.op_off = c.op_off;
        s.feat_off = bb.feat_per_cam ? c.row_off : c.op_off;
        s.pix_off = c.pix_off;
    } else {
        const int gxn = (W + kTile - 1) / kTile;
        s.W = W;
        s.H = H;
        s.P = P;
        s.tx = blockIdx.x;
        s.ty = blockIdx.y / SPLIT;
        s.part = blockIdx.y % SPLIT;
        s.tidx = s.ty * gxn + s.tx;
        s.row_off = s.op_off = s.feat_off = s.pix_off = 0;
    }
    return s;
}

constexpr int kBlendThreads = kTilePixels;  // 256: one thread per pixel
constexpr int kBatch = kBlendThreads;

// Register caps of the C <= 4 blend kernels (compile-time tunables; 0 = the
// compiler's choice): a cap of R registers asks for 65536 / (R x threads)
// resident blocks per SM.
#ifndef MSPLAT_BLEND_FWD_REGS
#define MSPLAT_BLEND_FWD_REGS 0
#endif
#ifndef MSPLAT_BLEND_BWD_REGS
#define MSPLAT_BLEND_BWD_REGS 0
#endif
// (Without a cap the kernels name no minimum block count at all: ptxas
// allocates differently for an explicit minimum of 1 -- 55 instead of 48
// registers in the forward, one block per SM fewer.)
#if MSPLAT_BLEND_FWD_REGS > 0
#define MSPLAT_FWD_BOUNDS(T) __launch_bounds__(T, 65536 / (MSPLAT_BLEND_FWD_REGS * (T)))
#else
#define MSPLAT_FWD_BOUNDS(T) __launch_bounds__(T)
#endif
#if MSPLAT_BLEND_BWD_REGS > 0
#define MSPLAT_BWD_BOUNDS(T) __launch_bounds__(T, 65536 / (MSPLAT_BLEND_BWD_REGS * (T)))
#else
#define MSPLAT_BWD_BOUNDS(T) __launch_bounds__(T)
#endif

struct BlendRec {
    float4 a;  // uv.x, uv.y, conic.x, conic.y
    float4 b;  // conic.z, opacity, power bound, list index (as int bits)
};


// Which warp blocks of a tile (or of the ROWS-row part of it a block
// renders) a Gaussian kept by the tile cull can reach.  The area is split
// into blocks 8 columns wide and RH rows tall, numbered
// 2 (row band) + (column half); bit w of the result covers block w.  Per
// column half [x0, x0 + 7] the reachable rows are the y-extent of the
// ellipse q <= L inside that band: the upper boundary
// y(x) = (-b x + sqrt(c L - det x^2)) / c is concave with its maximum
// sqrt(L a / det) at x = -b sqrt(L a / det) / a, so over the band it peaks
// there or at the nearer band edge (the lower boundary mirrors it); a band
// beyond the ellipse's x-extent sqrt(L c / det) is not reached at all.
// Extents are widened by 1 % plus 0.05 px and the coordinates' rounding,
// which covers their float evaluation (with det >= 0.01 a c the
// discriminant's rounding moves an extent by < 0.6 %); nearly degenerate
// conics (det < 0.01 a c), or no usable L, reach every block.  Skipping a
// block skips only pairs whose alpha is below 1/255: results do not change.
template <int RH, int ROWS = kTile>
__device__ __forceinline__ unsigned warp_block_mask(float gx, float gy, float a, float b, float c, float L,
                                                    float bx0, float by0) {
    constexpr int NBY = ROWS / RH;
    constexpr unsigned FULL = (1u << (2 * NBY)) - 1u;
    const float det = a * c - b * b;
    if (!(L >= 0.0f) || !(L < INFINITY) || !(a > 0.0f) || !(c > 0.0f) || !(det >= 0.01f * a * c))
        return FULL;
    const float ey = sqrtf(L * a / det), ex = sqrtf(L * c / det);
    const float xt = -b * ey / a;  // dx of the topmost point; the lowest is at -xt
    const float my = 0.01f * ey + 0.05f + 4e-6f * (fabsf(gy) + fabsf(by0) + (float)kTile);
    const float mx = 0.01f * ex + 0.05f + 4e-6f * (fabsf(gx) + fabsf(bx0) + (float)kTile);
    unsigned mask = 0u;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const float lx = bx0 + (float)(8 * h) - gx, hx = lx + 7.0f;
        if (hx < -ex - mx || lx > ex + mx) continue;  // band beyond the ellipse
        float top = ey, bot = -ey;
        if (!(xt >= lx && xt <= hx)) {
            const float x = fminf(fmaxf(xt, lx), hx);
            top = (-b * x + sqrtf(fmaxf(c * L - det * x * x, 0.0f))) / c;
        }
        if (!(-xt >= lx && -xt <= hx)) {
            const float x = fminf(fmaxf(-xt, lx), hx);
            bot = (-b * x - sqrtf(fmaxf(c * L - det * x * x, 0.0f))) / c;
        }
        const float lo = gy + bot - my - by0, hi = gy + top + my - by0;  // rows, pixel centres at by0 + r
        if (!(lo <= hi)) return FULL;
        if (hi < 0.0f || lo > (float)(ROWS - 1)) continue;
        const int glo = (int)floorf(fmaxf(lo, 0.0f)) / RH;
        const int ghi = (int)ceilf(fminf(hi, (float)(ROWS - 1))) / RH;
#pragma unroll
        for (int g = 0; g < NBY; ++g)
            if (g >= glo && g <= ghi) mask |= 1u << (2 * g + h);
    }
    return mask;
}

// power < bound  =>  opacity * exp(power) < 1/255 (with margin for the
// approximate exponential); -inf disables the shortcut.
__device__ __forceinline__ float power_bound(float op) {
    if (!(op > 0.0f)) return -INFINITY;
    const float h = -logf(255.0f * op);
    return h - (1e-3f + 1e-5f * fabsf(h));
}

// Gathers entry `j` (when valid) and compacts the kept entries of the block
// into shared memory in thread order.  Returns the number kept.
template <int CMAX>
__device__ __forceinline__ int gather_batch(bool valid, int j, int P, const int32_t *__restrict__ idx_sorted,
                                            const float2 *__restrict__ uv, const float *__restrict__ conic,
                                            const float *__restrict__ opacity,
                                            const float *__restrict__ feature, int C, int c0, int nc,
                                            float bx0, float by0, BlendRec *srec, float *sfeat,
                                            int *sgid, int *swarp) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    BlendRec r;
    int g = 0;
    bool keep = false;
    if (valid) g = idx_sorted[j];
    if (valid && (unsigned)g < (unsigned)P) {  // (an id outside the rows is never read)
        const float2 p = uv[g];
        const float ca = conic[3 * g], cb = conic[3 * g + 1], cc = conic[3 * g + 2];
        const float op = opacity[g];
        keep = !cull_tile(p.x, p.y, ca, cb, cc, op, bx0, by0);
        r.a = make_float4(p.x, p.y, ca, cb);
        r.b = make_float4(cc, op, power_bound(op), __int_as_float(j));
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) swarp[warp] = __popc(m);
    __syncthreads();
    int base = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kBlendThreads / 32; ++w) {
        const int cw = swarp[w];
        base += (w < warp) ? cw : 0;
        total += cw;
    }
    if (keep) {
        const int pos = base + __popc(m & ((1u << lane) - 1u));
        srec[pos] = r;
        sgid[pos] = g;
        const float *f = feature + (size_t)g * C + c0;
#pragma unroll
        for (int k = 0; k < CMAX; ++k)
            if (k < nc) sfeat[k * kBatch + pos] = f[k];
    }
    __syncthreads();
    return total;
}

template <int CMAX, bool BATCH = false>
__global__ void __launch_bounds__(kBlendThreads)
blend_fwd_kernel(int P, int C, int c0, const float2 *__restrict__ uv, const float *__restrict__ conic,
                 const float *__restrict__ opacity, const float *__restrict__ feature,
                 const int32_t *__restrict__ idx_sorted, const int2 *__restrict__ tile_range, float bg,
                 int W, int H, float *__restrict__ out, float *__restrict__ final_T,
                 int32_t *__restrict__ ncontrib, BlendBatch bb = {}) {
    __shared__ BlendRec srec[kBatch];
    extern __shared__ float sfeat[];  // [CMAX][kBatch] (dynamic: up to 64 KB)
    __shared__ int sgid[kBatch];
    __shared__ int swarp[kBlendThreads / 32];
    const int nc = min(CMAX, C - c0);
    const BlendSite site = blend_site<BATCH, 1>(bb, P, W, H);
    if (BATCH) {
        W = site.W;
        H = site.H;
        uv += site.row_off;
        conic += 3 * site.row_off;
        opacity += site.op_off;
        feature += (size_t)C * site.feat_off;
        out += (size_t)C * site.pix_off;
        final_T += site.pix_off;
        ncontrib += site.pix_off;
    }
    const int px = site.tx * kTile + (threadIdx.x & (kTile - 1));
    const int py = site.ty * kTile + (threadIdx.x >> 4);
    const bool inside = px < W && py < H;
    const float fx = (float)px, fy = (float)py;
    const float bx0 = (float)(site.tx * kTile), by0 = (float)(site.ty * kTile);
    const int2 range = tile_range[site.tidx];

    bool done = !inside;
    float T = 1.0f;
    int last = 0;
    float F[CMAX];
#pragma unroll
    for (int k = 0; k < CMAX; ++k) F[k] = 0.0f;

    for (int start = range.x; start < range.y; start += kBatch) {
        if (__syncthreads_count(done) == kBlendThreads) break;
        const int j = start + (int)threadIdx.x;
        const int n = gather_batch<CMAX>(j < range.y, j, site.P, idx_sorted, uv, conic, opacity, feature, C, c0,
                                         nc, bx0, by0, srec, sfeat, sgid, swarp);
        for (int k = 0; k < n && !done; ++k) {
            const BlendRec r = srec[k];
            const float dx = r.a.x - fx, dy = r.a.y - fy;
            const float power = -0.5f * (r.a.z * dx * dx + r.b.x * dy * dy) - r.a.w * dx * dy;
            if (power > 0.0f || power < r.b.z) continue;
            const float alpha = fminf(0.99f, r.b.y * __expf(power));
            if (alpha < 1.0f / 255.0f) continue;
            const float nT = T * (1.0f - alpha);
            if (nT < 0.0001f) {
                done = true;
                continue;
            }
            const float at = alpha * T;  // as the C <= 4 walk: f (alpha T)
#pragma unroll
            for (int q = 0; q < CMAX; ++q)
                if (q < nc) F[q] += sfeat[q * kBatch + k] * at;
            T = nT;
            last = __float_as_int(r.b.w) - range.x + 1;
        }
    }
    if (inside) {
        const int pix = py * W + px;
        if (c0 == 0) {
            final_T[pix] = T;
            ncontrib[pix] = last;
        }
#pragma unroll
        for (int q = 0; q < CMAX; ++q)
            if (q < nc) out[(size_t)(c0 + q) * H * W + pix] = F[q] + T * bg;
    }
}

// Reduce-scatter of 16 values over a warp: lane l returns the warp total of
// value (l >> 1) (lanes 2i and 2i+1 hold the same total).
__device__ __forceinline__ float warp_reduce_scatter16(float (&v)[16]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16, n = 16; o >= 2; o >>= 1, n >>= 1) {
        const bool up = (lane & o) != 0;
        const int h = n >> 1;
#pragma unroll
        for (int k = 0; k < h; ++k) {
            const float send = up ? v[k] : v[k + h];
            const float keep = up ? v[k + h] : v[k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

constexpr int kBwdC = 10;  // channels per backward pass (6 + 10 = 16 values)

template <bool BATCH = false>
__global__ void __launch_bounds__(kBlendThreads)
blend_bwd_kernel(int P, int C, int c0, const float2 *__restrict__ uv, const float *__restrict__ conic,
                 const float *__restrict__ opacity, const float *__restrict__ feature,
                 const int32_t *__restrict__ idx_sorted, const int2 *__restrict__ tile_range, float bg,
                 int W, int H, const float *__restrict__ final_T, const int32_t *__restrict__ ncontrib,
                 const float *__restrict__ dL_dout, float *__restrict__ dL_duv,
                 float *__restrict__ dL_dconic, float *__restrict__ dL_dopacity,
                 float *__restrict__ dL_dfeature, BlendBatch bb = {}) {
    __shared__ BlendRec srec[kBatch];
    __shared__ float sfeat[kBwdC * kBatch];
    __shared__ int sgid[kBatch];
    __shared__ int swarp[kBlendThreads / 32];
    __shared__ int smax;
    const int nc = min(kBwdC, C - c0);
    const BlendSite site = blend_site<BATCH, 1>(bb, P, W, H);
    if (BATCH) {
        W = site.W;
        H = site.H;
        uv += site.row_off;
        conic += 3 * site.row_off;
        opacity += site.op_off;
        feature += (size_t)C * site.feat_off;
        final_T += site.pix_off;
        ncontrib += site.pix_off;
        dL_dout += (size_t)C * site.pix_off;
        dL_duv += 2 * site.row_off;
        dL_dconic += 3 * site.row_off;
        dL_dopacity += site.row_off;
        dL_dfeature += (size_t)C * site.row_off;
    }
    const int px = site.tx * kTile + (threadIdx.x & (kTile - 1));
    const int py = site.ty * kTile + (threadIdx.x >> 4);
    const bool inside = px < W && py < H;
    const float fx = (float)px, fy = (float)py;
    const float bx0 = (float)(site.tx * kTile), by0 = (float)(site.ty * kTile);
    const int2 range = tile_range[site.tidx];
    const int pix = py * W + px;
    const int lane = threadIdx.x & 31;

    const float T_final = inside ? final_T[pix] : 0.0f;
    const int last = inside ? ncontrib[pix] : 0;
    float T = T_final;
    float dpix[kBwdC], accum[kBwdC], lastf[kBwdC];
    float bg_dot = 0.0f;
#pragma unroll
    for (int q = 0; q < kBwdC; ++q) {
        dpix[q] = (inside && q < nc) ? dL_dout[(size_t)(c0 + q) * H * W + pix] : 0.0f;
        accum[q] = 0.0f;
        lastf[q] = 0.0f;
        bg_dot += bg * dpix[q];
    }
    float last_alpha = 0.0f;

    // Nothing past the tile's largest ncontrib contributes.
    if (threadIdx.x == 0) smax = 0;
    __syncthreads();
    int wmax = last;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
    if (lane == 0) atomicMax(&smax, wmax);
    __syncthreads();
    const int end = range.x + min(smax, range.y - range.x);

    for (int bend = end; bend > range.x; bend -= kBatch) {
        const int bstart = max(range.x, bend - kBatch);
        const int j = bend - 1 - (int)threadIdx.x;
        const int n = gather_batch<kBwdC>(j >= bstart, j, site.P, idx_sorted, uv, conic, opacity, feature, C, c0,
                                          nc, bx0, by0, srec, sfeat, sgid, swarp);
        for (int k = 0; k < n; ++k) {
            const BlendRec r = srec[k];
            const int jl = __float_as_int(r.b.w) - range.x;  // list position
            float v[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) v[q] = 0.0f;
            bool contrib = false;
            if (jl < last) {
                const float dx = r.a.x - fx, dy = r.a.y - fy;
                const float ca = r.a.z, cb = r.a.w, cc = r.b.x, op = r.b.y;
                const float power = -0.5f * (ca * dx * dx + cc * dy * dy) - cb * dx * dy;
                if (power <= 0.0f && power >= r.b.z) {
                    const float G = __expf(power);
                    const float alpha = fminf(0.99f, op * G);
                    if (alpha >= 1.0f / 255.0f) {
                        contrib = true;
                        T = T / (1.f - alpha);
                        const float dcol = alpha * T;
                        float dL_dalpha = 0.0f;
#pragma unroll
                        for (int q = 0; q < kBwdC; ++q) {
                            if (q < nc) {
                                const float f = sfeat[q * kBatch + k];
                                accum[q] = last_alpha * lastf[q] + (1.f - last_alpha) * accum[q];
                                lastf[q] = f;
                                dL_dalpha += (f - accum[q]) * dpix[q];
                                v[6 + q] = dcol * dpix[q];
                            }
                        }
                        dL_dalpha *= T;
                        last_alpha = alpha;
                        dL_dalpha += (-T_final / (1.f - alpha)) * bg_dot;
                        const float dL_dG = op * dL_dalpha;
                        const float gdx = -G * dx * ca - G * dy * cb;
                        const float gdy = -G * dy * cc - G * dx * cb;
                        v[0] = dL_dG * gdx;
                        v[1] = dL_dG * gdy;
                        v[2] = -0.5f * G * dx * dx * dL_dG;
                        v[3] = -G * dx * dy * dL_dG;
                        v[4] = -0.5f * G * dy * dy * dL_dG;
                        v[5] = G * dL_dalpha;
                    }
                }
            }
            if (__any_sync(0xffffffffu, contrib)) {
                const float s = warp_reduce_scatter16(v);
                const int vi = lane >> 1;
                if ((lane & 1) == 0 && vi < 6 + nc) {
                    const int g = sgid[k];
                    float *dst;
                    if (vi < 2) dst = dL_duv + 2 * g + vi;
                    else if (vi < 5) dst = dL_dconic + 3 * g + (vi - 2);
                    else if (vi == 5) dst = dL_dopacity + g;
                    else dst = dL_dfeature + (size_t)g * C + c0 + (vi - 6);
                    atomicAdd(dst, s);
                }
            }
        }
        __syncthreads();
    }
}


// ===================================================================
// Backward for 4 < C <= CMAX channels in one walk.  The pair's geometry, its
// transmittance and the colour recursion are evaluated once per pair for
// all channels -- the recursion carried as two scalars, as in the C <= 4
// kernels (the reference's per-channel accum_rec enters dL/dalpha only
// through its dot product with dL/dpix) -- and the gradients go out in
// groups of 16 values per warp reduce-scatter: the six geometry gradients
// with the first 10 colour channels, then 16 channels at a time.  (Walking
// the list once per 10 channels, as blend_bwd_kernel does, repeats the
// pair's geometry and recursion per chunk.)  A pixel past its last
// contributor, or where the pair's alpha is below 1/255, adds zeros.
// ===================================================================
template <int CMAX>
inline size_t blend_bwd_wide_smem() {
    return (size_t)kBatch * (sizeof(BlendRec) + sizeof(int)) + (size_t)CMAX * kBatch * sizeof(float);
}

template <int CMAX, bool BATCH = false>
__global__ void __launch_bounds__(kBlendThreads)
blend_bwd_wide_kernel(int P, int C, const float2 *__restrict__ uv, const float *__restrict__ conic,
                      const float *__restrict__ opacity, const float *__restrict__ feature,
                      const int32_t *__restrict__ idx_sorted, const int2 *__restrict__ tile_range, float bg, int W,
                      int H, const float *__restrict__ final_T, const int32_t *__restrict__ ncontrib,
                      const float *__restrict__ dL_dout, float *__restrict__ dL_duv, float *__restrict__ dL_dconic,
                      float *__restrict__ dL_dopacity, float *__restrict__ dL_dfeature, BlendBatch bb) {
    extern __shared__ __align__(16) unsigned char wide_raw[];
    BlendRec *srec = reinterpret_cast<BlendRec *>(wide_raw);
    int *sgid = reinterpret_cast<int *>(srec + kBatch);
    float *sfeat = reinterpret_cast<float *>(sgid + kBatch);  // [CMAX][kBatch]
    __shared__ int swarp[kBlendThreads / 32];
    __shared__ int smax;
    const BlendSite site = blend_site<BATCH, 1>(bb, P, W, H);
    if (BATCH) {
        W = site.W;
        H = site.H;
        uv += site.row_off;
        conic += 3 * site.row_off;
        opacity += site.op_off;
        feature += (size_t)C * site.feat_off;
        final_T += site.pix_off;
        ncontrib += site.pix_off;
        dL_dout += (size_t)C * site.pix_off;
        dL_duv += 2 * site.row_off;
        dL_dconic += 3 * site.row_off;
        dL_dopacity += site.row_off;
        dL_dfeature += (size_t)C * site.row_off;
    }
    const int px = site.tx * kTile + (threadIdx.x & (kTile - 1));
    const int py = site.ty * kTile + (threadIdx.x >> 4);
    const bool inside = px < W && py < H;
    const float fx = (float)px, fy = (float)py;
    const float bx0 = (float)(site.tx * kTile), by0 = (float)(site.ty * kTile);
    const int2 range = tile_range[site.tidx];
    const int pix = py * W + px;
    const int lane = threadIdx.x & 31;

    const float T_final = inside ? final_T[pix] : 0.0f;
    const int last = inside ? ncontrib[pix] : 0;
    float T = T_final, ad = 0.0f, lfd = 0.0f, la = 0.0f;
    float dpix[CMAX];
    float bg_dot = 0.0f;
#pragma unroll
    for (int q = 0; q < CMAX; ++q) {
        dpix[q] = (inside && q < C) ? dL_dout[(size_t)q * H * W + pix] : 0.0f;
        bg_dot += bg * dpix[q];
    }

    // Nothing past the tile's largest ncontrib contributes.
    if (threadIdx.x == 0) smax = 0;
    __syncthreads();
    int wmax = last;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
    if (lane == 0) atomicMax(&smax, wmax);
    __syncthreads();
    const int end = range.x + min(smax, range.y - range.x);

    for (int bend = end; bend > range.x; bend -= kBatch) {
        const int bstart = max(range.x, bend - kBatch);
        const int j = bend - 1 - (int)threadIdx.x;
        const int n = gather_batch<CMAX>(j >= bstart, j, site.P, idx_sorted, uv, conic, opacity, feature, C, 0, C,
                                         bx0, by0, srec, sfeat, sgid, swarp);
        for (int k = 0; k < n; ++k) {
            const BlendRec r = srec[k];
            const int jl = __float_as_int(r.b.w) - range.x;  // list position
            const float dx = r.a.x - fx, dy = r.a.y - fy;
            const float ca = r.a.z, cb = r.a.w, cc = r.b.x, op = r.b.y;
            const float power = -0.5f * (ca * dx * dx + cc * dy * dy) - cb * dx * dy;
            const float G = __expf(power);
            const float alpha = fminf(0.99f, op * G);
            const bool ok = jl < last && power <= 0.0f && !(alpha < 1.0f / 255.0f);
            if (!__any_sync(0xffffffffu, ok)) continue;
            const float inv1m = __fdividef(1.f, 1.f - alpha);
            const float Tn = T * inv1m;
            const float dcol = ok ? alpha * Tn : 0.0f;
            float fd = 0.0f;  // colour . dL/dpix
#pragma unroll
            for (int q = 0; q < CMAX; ++q)
                if (q < C) fd += sfeat[q * kBatch + k] * dpix[q];
            const float adn = la * lfd + (1.f - la) * ad;
            float dL_dalpha = (fd - adn) * Tn;
            dL_dalpha += (-T_final * inv1m) * bg_dot;
            const float dL_dG = ok ? op * dL_dalpha : 0.0f;
            const float gdx = -G * dx * ca - G * dy * cb;
            const float gdy = -G * dy * cc - G * dx * cb;
            float v[16];
            v[0] = dL_dG * gdx;
            v[1] = dL_dG * gdy;
            v[2] = -0.5f * G * dx * dx * dL_dG;
            v[3] = -G * dx * dy * dL_dG;
            v[4] = -0.5f * G * dy * dy * dL_dG;
            v[5] = ok ? G * dL_dalpha : 0.0f;
#pragma unroll
            for (int i = 0; i < 10; ++i) v[6 + i] = dcol * dpix[i];
            T = ok ? Tn : T;
            ad = ok ? adn : ad;
            lfd = ok ? fd : lfd;
            la = ok ? alpha : la;
            const int g = sgid[k];
            {
                const float s = warp_reduce_scatter16(v);
                const int vi = lane >> 1;
                if ((lane & 1) == 0 && vi < 6 + min(10, C)) {
                    float *dst;
                    if (vi < 2) dst = dL_duv + 2 * g + vi;
                    else if (vi < 5) dst = dL_dconic + 3 * g + (vi - 2);
                    else if (vi == 5) dst = dL_dopacity + g;
                    else dst = dL_dfeature + (size_t)g * C + (vi - 6);
                    atomicAdd(dst, s);
                }
            }
#pragma unroll
            for (int q0 = 10; q0 < CMAX; q0 += 16) {
                if (q0 < C) {  // (uniform)
                    float w[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) w[i] = q0 + i < CMAX ? dcol * dpix[q0 + i] : 0.0f;
                    const float s = warp_reduce_scatter16(w);
                    const int vi = lane >> 1;
                    if ((lane & 1) == 0 && q0 + vi < C) atomicAdd(dL_dfeature + (size_t)g * C + q0 + vi, s);
                }
            }
        }
        __syncthreads();
    }
}

// ===================================================================
// Several pixels per thread, C <= 4 channels (the common RGB case).
//
// A thread owns NPIX pixels of one tile column (rows ly, ly + 16/NPIX, ...),
// so each gathered Gaussian is read from shared memory once per NPIX pixels
// and, in the backward, the per-Gaussian sums over a warp cover 32 * NPIX
// pixels per reduction.  Pairs of pixels are evaluated with packed f32x2
// arithmetic.  The reference's per-pair expression
//   power = -0.5f * (a*dx*dx + c*dy*dy) - b*dx*dy
// is spelled out with the FMA contractions the compiler gives it in the
// one-pixel kernels above (the product a*dx*dx fused into the sum, b*dx*dy
// fused into the scaling), so every pixel sees bit-identical powers,
// alphas, transmittances and contributor counts.
// ===================================================================

template <int NPIX>
struct PixPow {
    float v[NPIX];
};

template <int NPIX>
__device__ __forceinline__ PixPow<NPIX> blend_power_n(float a, float b, float c, float dx,
                                                      const float (&dy)[NPIX]) {
    PixPow<NPIX> out;
    const float adx = __fmul_rn(a, dx), bdx = __fmul_rn(b, dx);
#pragma unroll
    for (int i = 0; i < NPIX; i += 2) {
        if (i + 1 < NPIX) {
            const float2 d = make_float2(dy[i], dy[i + 1]);
            const float2 cdd = __fmul2_rn(__fmul2_rn(make_float2(c, c), d), d);
            const float2 s = __ffma2_rn(make_float2(adx, adx), make_float2(dx, dx), cdd);
            const float2 bdd = __fmul2_rn(make_float2(bdx, bdx), d);
            const float2 pw = __ffma2_rn(make_float2(-0.5f, -0.5f), s, make_float2(-bdd.x, -bdd.y));
            out.v[i] = pw.x;
            out.v[i + 1] = pw.y;
        } else {
            const float s = __fmaf_rn(adx, dx, __fmul_rn(__fmul_rn(c, dy[i]), dy[i]));
            out.v[i] = __fmaf_rn(-0.5f, s, -__fmul_rn(bdx, dy[i]));
        }
    }
    return out;
}

// The warp-block masks of a tile list's entries, as the forward computed
// them, kept for the backward: emask[j] for list position j holds the
// blocks of 8 columns by 4 NPB rows (the backward's warp blocks) entry j
// can reach (0: the tile cull dropped it).  The forward writes them (out)
// for every position it gathers -- every position up to the tile's last
// contributor -- and the backward reads them (in) instead of repeating the
// cull and mask arithmetic.  Either pointer may be null.
struct EntryMasks {
    const unsigned char *__restrict__ in = nullptr;
    unsigned char *__restrict__ out = nullptr;
};

// A mask of warp blocks of RF rows as one of blocks of RT rows (RT a
// multiple of RF): block g of RT rows covers blocks g K .. g K + K - 1.
template <int RF, int RT, int ROWS>
__device__ __forceinline__ unsigned merge_block_rows(unsigned m) {
    constexpr int K = RT / RF, NB = ROWS / RT;
    if (K == 1) return m;
    unsigned out = 0u;
#pragma unroll
    for (int g = 0; g < NB; ++g)
#pragma unroll
        for (int k = 0; k < K; ++k) out |= ((m >> (2 * (g * K + k))) & 3u) << (2 * g);
    return out;
}

// One entry of a tile's list: its record (uv, conic, opacity, list index),
// features and warp-block mask, and whether the tile cull (the box of ROWS
// rows from by0) keeps it.  (No power bound: the branch-free walks evaluate
// every pair's alpha, which the bound only let them skip.)  With em.in the
// mask comes from there (kept: mask != 0) and no cull is evaluated; with
// em.out the entry's mask in the geometry of NPB pixels per thread is
// stored there.
template <int C, int NPIX, int ROWS, int NPB = NPIX>
__device__ __forceinline__ bool gather_entry(int j, int P, const int32_t *__restrict__ idx_sorted,
                                             const float2 *__restrict__ uv, const float *__restrict__ conic,
                                             const float *__restrict__ opacity, const float *__restrict__ feature,
                                             float bx0, float by0, float4 &A, float4 &B, float4 &F, int &G,
                                             unsigned &M, EntryMasks em = {}) {
    const int g = idx_sorted[j];
    unsigned mi = 1u;
    if (em.in) mi = em.in[j];
    if ((unsigned)g >= (unsigned)P || mi == 0u) {  // an id outside the rows is never read
        A = B = F = make_float4(0.f, 0.f, 0.f, 0.f);
        G = 0;
        M = 0u;
        if (em.out) em.out[j] = 0;
        return false;
    }
    const float2 p = uv[g];
    const float ca = conic[3 * g], cb = conic[3 * g + 1], cc = conic[3 * g + 2];
    const float op = opacity[g];
    bool keep;
    if (em.in) {
        keep = true;
        M = mi;
    } else {
        float L;
        keep = !cull_box(p.x, p.y, ca, cb, cc, op, bx0, by0, bx0 + (float)(kTile - 1), by0 + (float)(ROWS - 1),
                         L);
        M = keep ? warp_block_mask<4 * NPIX, ROWS>(p.x, p.y, ca, cb, cc, L, bx0, by0) : 0u;
        if (em.out) {
            unsigned mo;
            if (NPB % NPIX == 0) mo = merge_block_rows<4 * NPIX, 4 * NPB, ROWS>(M);
            else mo = keep ? warp_block_mask<4 * NPB, ROWS>(p.x, p.y, ca, cb, cc, L, bx0, by0) : 0u;
            em.out[j] = (unsigned char)mo;
        }
    }
    A = make_float4(p.x, p.y, ca, cb);
    B = make_float4(cc, op, 0.0f, __int_as_float(j));  // (z unused: the walks evaluate every alpha)
    float f[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < C; ++q) f[q] = feature[(size_t)g * C + q];
    F = make_float4(f[0], f[1], f[2], f[3]);
    G = g;
    return keep;
}

// Gathers GE entries per thread (thread t owns list positions
// base + dir * (t * GE + r)) and compacts the kept ones into shared
// memory in list order, with the mask of the warp blocks (8 columns by
// 4 NPIX rows, one per warp) each one can reach.  The block renders the
// ROWS rows from by0 of the tile, which is also the box of the cull.
// Returns the number kept, or -1 (nothing written) when every thread's
// `vote` is set.
// Its first barrier is the only one between two batches: shared records
// are written after it, and every warp reaches it only once done with the
// previous batch, so a warp that finishes a batch early issues the next
// batch's loads and cull tests while the others still blend.
template <int C, int NPIX, bool WITH_ID, int ROWS = kTile, int GE = NPIX, int NPB = NPIX>
__device__ __forceinline__ int gather_small(int base, int dir, int lo, int hi, int P,
                                            const int32_t *__restrict__ idx_sorted,
                                            const float2 *__restrict__ uv, const float *__restrict__ conic,
                                            const float *__restrict__ opacity,
                                            const float *__restrict__ feature, float bx0, float by0,
                                            float4 *sA, float4 *sB, float4 *sF, int *sG, unsigned char *sM,
                                            int *scan, bool vote, EntryMasks em = {}) {
    constexpr int NT = kTile * ROWS / NPIX;
    float4 A[GE], B[GE], F[GE];
    int G[GE];
    unsigned M[GE];
    bool keep[GE];
    int nk = 0;
#pragma unroll
    for (int r = 0; r < GE; ++r) {
        const int j = base + dir * ((int)threadIdx.x * GE + r);
        keep[r] = false;
        if (j >= lo && j < hi)
            keep[r] = gather_entry<C, NPIX, ROWS, NPB>(j, P, idx_sorted, uv, conic, opacity, feature, bx0, by0, A[r],
                                                       B[r], F[r], G[r], M[r], em);
        nk += keep[r];
    }
    // Block exclusive scan of the per-thread counts (NT <= 256 threads).
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = nk;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += n;
    }
    if (lane == 31) scan[warp] = inc;
    if (__syncthreads_count(vote) == NT) return -1;
    int wbase = 0, total = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) {
        const int c = scan[w];
        wbase += (w < warp) ? c : 0;
        total += c;
    }
    int pos = wbase + inc - nk;
#pragma unroll
    for (int r = 0; r < GE; ++r) {
        if (keep[r]) {
            sA[pos] = A[r];
            sB[pos] = B[r];
            sF[pos] = F[r];
            sM[pos] = (unsigned char)M[r];
            if (WITH_ID) sG[pos] = G[r];
            ++pos;
        }
    }
    __syncthreads();
    return total;
}

// The forward's walk over one gathered batch of n entries: each warp walks,
// 32 entries at a time, only the entries whose warp-block mask has its bit
// (a warp-uniform bit set from one ballot), and leaves the batch once all
// of its pixels are done (tested before each 32 entries; a done pixel takes
// no further update).  list0: the list index of the tile's first entry.
// The per-pixel step has no branch: every pixel evaluates the entry and
// keeps the result only where the reference's tests (alpha >= 1/255, T
// stays >= 1e-4) pass -- the same values, selected instead of branched
// around (measured 7 % faster than the branching walk at 1M / 1080p).  The
// colour adds f (alpha T) with alpha T formed once (the reference forms
// (f alpha) T: the two differ by rounding only, 5 % faster).
template <int C, int NPIX>
__device__ __forceinline__ void fwd_walk_batch(int n, const float4 *sA, const float4 *sB, const float4 *sF,
                                               const unsigned char *sM, unsigned wbit, float fx,
                                               const float (&fy)[NPIX], bool (&done)[NPIX], float (&T)[NPIX],
                                               float (&F)[NPIX][4], int (&last)[NPIX], int list0) {
    const int lane = threadIdx.x & 31;
    for (int kw = 0; kw < n; kw += 32) {
        bool ad = true;
#pragma unroll
        for (int i = 0; i < NPIX; ++i) ad &= done[i];
        if (__all_sync(0xffffffffu, ad)) return;
        unsigned bits = __ballot_sync(0xffffffffu, kw + lane < n && (sM[kw + lane] & wbit));
        while (bits) {
            const int k = kw + __ffs(bits) - 1;
            bits &= bits - 1u;
            const float4 A = sA[k], B = sB[k];
            const float dx = A.x - fx;
            float dy[NPIX];
#pragma unroll
            for (int i = 0; i < NPIX; ++i) dy[i] = A.y - fy[i];
            const PixPow<NPIX> pw = blend_power_n<NPIX>(A.z, A.w, B.x, dx, dy);
            const float4 f = sF[k];
            const float fv[4] = {f.x, f.y, f.z, f.w};
            const int id1 = __float_as_int(B.w) - list0 + 1;
#pragma unroll
            for (int i = 0; i < NPIX; ++i) {
                const float power = pw.v[i];
                const bool skip = done[i] || power > 0.0f;
                const float alpha = fminf(0.99f, B.y * __expf(power));
                const float nT = T[i] * (1.0f - alpha);
                const bool use = !skip && !(alpha < 1.0f / 255.0f);
                const bool fin = use && nT < 0.0001f;  // the pixel ends before this entry
                const bool upd = use && !fin;
                const float at = alpha * T[i];
#pragma unroll
                for (int q = 0; q < C; ++q) {
                    const float nf = F[i][q] + fv[q] * at;
                    F[i][q] = upd ? nf : F[i][q];
                }
                T[i] = upd ? nT : T[i];
                last[i] = upd ? id1 : last[i];
                done[i] = done[i] || fin;
            }
        }
    }
}

// SPLIT: a tile is rendered by SPLIT blocks of kTile / SPLIT rows each
// (grid.y = tiles down x SPLIT), each gathering the tile's list against
// its own part.
template <int C, int NPIX, int SPLIT, bool BATCH = false, int GE = NPIX, int NPB = NPIX>
__global__ void MSPLAT_FWD_BOUNDS(kTilePixels / NPIX / SPLIT)
blend_fwd_small_kernel(int P, const float2 *__restrict__ uv, const float *__restrict__ conic,
                       const float *__restrict__ opacity, const float *__restrict__ feature,
                       const int32_t *__restrict__ idx_sorted, const int2 *__restrict__ tile_range, float bg,
                       int W, int H, float *__restrict__ out, float *__restrict__ final_T,
                       int32_t *__restrict__ ncontrib, unsigned char *__restrict__ emask, BlendBatch bb) {
    static_assert(!BATCH || SPLIT == 1, "batched blends render whole tiles");
    // GE entries gathered per thread: BATCH_N Gaussians per shared-memory batch
    constexpr int ROWS = kTile / SPLIT, NT = kTile * ROWS / NPIX, BATCH_N = NT * GE;
    static_assert(4 * NPIX <= ROWS, "a warp block of 4 NPIX rows must fit the block's rows");
    __shared__ float4 sA[BATCH_N], sB[BATCH_N], sF[BATCH_N];
    __shared__ unsigned char sM[BATCH_N];
    __shared__ int scan[NT / 32];
    const BlendSite site = blend_site<BATCH, SPLIT>(bb, P, W, H);
    if (BATCH) {
        W = site.W;
        H = site.H;
        uv += site.row_off;
        conic += 3 * site.row_off;
        opacity += site.op_off;
        feature += (size_t)C * site.feat_off;
        out += (size_t)C * site.pix_off;
        final_T += site.pix_off;
        ncontrib += site.pix_off;
    }
    const int2 range = tile_range[site.tidx];
    // warp w owns the block of 8 columns (8 (w % 2) ...) by 4 NPIX rows
    // (4 NPIX (w / 2) ...) that bit w of a gathered entry's mask covers;
    // lane l takes column l % 8 and rows (l / 8) NPIX + i of it
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row0 = site.ty * kTile + site.part * ROWS;
    const int px = site.tx * kTile + 8 * (warp & 1) + (lane & 7);
    const int py0 = row0 + 4 * NPIX * (warp >> 1) + (lane >> 3) * NPIX;
    const unsigned wbit = 1u << warp;
    const float fx = (float)px;
    const float bx0 = (float)(site.tx * kTile), by0 = (float)row0;
    float fy[NPIX], T[NPIX], F[NPIX][4];
    int last[NPIX];
    bool done[NPIX];
#pragma unroll
    for (int i = 0; i < NPIX; ++i) {
        const int py = py0 + i;
        fy[i] = (float)py;
        T[i] = 1.0f;
        last[i] = 0;
        done[i] = !(px < W && py < H);
#pragma unroll
        for (int q = 0; q < 4; ++q) F[i][q] = 0.0f;
    }
    for (int start = range.x; start < range.y; start += BATCH_N) {
        bool all_done = true;
#pragma unroll
        for (int i = 0; i < NPIX; ++i) all_done &= done[i];
        const int n = gather_small<C, NPIX, false, ROWS, GE, NPB>(start, 1, range.x, range.y, site.P, idx_sorted, uv,
                                                              conic, opacity, feature, bx0, by0, sA, sB, sF, nullptr,
                                                              sM, scan, all_done, EntryMasks{nullptr, emask});
        if (n < 0) break;  // every pixel of the block is done
        fwd_walk_batch<C, NPIX>(n, sA, sB, sF, sM, wbit, fx, fy, done, T, F, last, range.x);
    }
#pragma unroll
    for (int i = 0; i < NPIX; ++i) {
        const int py = py0 + i;
        if (px < W && py < H) {
            const int pix = py * W + px;
            final_T[pix] = T[i];
            ncontrib[pix] = last[i];
#pragma unroll
            for (int q = 0; q < C; ++q) out[(size_t)q * H * W + pix] = F[i][q] + T[i] * bg;
        }
    }
}

// ===================================================================
// Forward blend as a producer / consumer ring (C <= 4, NPIX pixels per
// consumer thread).
//
// NP producer warps gather, cull and mask each 256-entry batch of a tile's
// list (the same per-entry work as gather_small), each compacting its share
// in list order into its own part of one of two shared-memory slots; the
// 8 / NPIX consumer warps (NPIX pixels per thread, the warp blocks of
// blend_fwd_small_kernel) blend a slot while the producers fill the other.  The hand-off is two mbarriers per slot: "full"
// (the producers' threads arrive once their records are written) and
// "empty" (each consumer warp arrives once done with the slot), so there is
// no block-wide barrier between batches and consumer warps with little work
// in a batch run on into the next one.  The producers stop at the end of
// the list or once every consumer warp's pixels are done (a shared count),
// and publish an end marker.  Results equal blend_fwd_small_kernel's bit
// for bit (same entries in the same order, same per-pair code).
//
// Every wait is bounded: after `wait_limit` polls (each suspends for at most
// kWaitHintNs) the thread sets the device error word g_wait_error and
// leaves its loop, so a lost hand-off ends the kernel with an error the
// host reads (msplat_wait_error) instead of a hang.
// ===================================================================

// Minimum resident ring blocks per SM (compile-time tunable; 0 = the
// compiler's choice).
#ifndef MSPLAT_RING_MIN_BLOCKS
#define MSPLAT_RING_MIN_BLOCKS 0
#endif
#if MSPLAT_RING_MIN_BLOCKS > 0
#define MSPLAT_RING_BOUNDS(T) __launch_bounds__(T, MSPLAT_RING_MIN_BLOCKS)
#else
#define MSPLAT_RING_BOUNDS(T) __launch_bounds__(T)
#endif

static __device__ int g_wait_error;  // 1 after a bounded wait of a blend gave up
constexpr uint32_t kWaitHintNs = 1000;
#ifndef MSPLAT_WAIT_LIMIT
#define MSPLAT_WAIT_LIMIT (1 << 21)  // polls of <= 1 us each: about 2 s at most
#endif
static int g_wait_limit = MSPLAT_WAIT_LIMIT;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ uint32_t mbar_try_wait(uint32_t addr, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(addr), "r"(parity), "r"(kWaitHintNs)
        : "memory");
    return ok;
}

// One thread waits for the completion of the barrier's phase of parity
// `parity`; false (and the error word set) after `limit` polls.
__device__ __forceinline__ bool mbar_wait_one(uint64_t *bar, uint32_t parity, int limit) {
    const uint32_t a = smem_u32(bar);
    for (int it = 0; it < limit; ++it)
        if (mbar_try_wait(a, parity)) return true;
    atomicExch(&g_wait_error, 1);
    return false;
}

// The whole warp waits (every lane polls, so every lane acquires the
// producers' writes), and the outcome is the same in every lane: a phase
// stays complete until this warp itself takes part in the next one, so once
// any lane sees it, all do within an iteration.  Bounded by `limit` polls.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t *bar, uint32_t parity, int limit) {
    const uint32_t a = smem_u32(bar);
    for (int it = 0; it < limit; ++it)
        if (__all_sync(0xffffffffu, mbar_try_wait(a, parity) != 0)) return true;
    if ((threadIdx.x & 31) == 0) atomicExch(&g_wait_error, 1);
    return false;
}

// Barrier 1 among the NP producer warps only (the consumers never use it).
template <int NP>
__device__ __forceinline__ void producer_sync() {
    asm volatile("bar.sync 1, %0;" ::"n"(NP * 32) : "memory");
}

template <int C, int NP, bool BATCH = false, int NPIX = 1, int NPB = NPIX>
__global__ void MSPLAT_RING_BOUNDS(kTilePixels / NPIX + 32 * NP)
blend_fwd_ring_kernel(int P, const float2 *__restrict__ uv, const float *__restrict__ conic,
                      const float *__restrict__ opacity, const float *__restrict__ feature,
                      const int32_t *__restrict__ idx_sorted, const int2 *__restrict__ tile_range, float bg, int W,
                      int H, float *__restrict__ out, float *__restrict__ final_T, int32_t *__restrict__ ncontrib,
                      unsigned char *__restrict__ emask, BlendBatch bb, int wait_limit) {
    constexpr int NC = kTilePixels / NPIX / 32;  // consumer warps (NPIX pixels per thread)
    constexpr int SLOT = kTilePixels;          // entries per batch
    constexpr int SUB = SLOT / NP;             // entries per producer warp (its own part of the slot)
    constexpr int PER = SUB / 32;              // gather rounds per producer warp
    static_assert(SLOT % (32 * NP) == 0, "producer warps must split a batch evenly");
    __shared__ float4 sA[2][SLOT], sB[2][SLOT], sF[2][SLOT];
    __shared__ unsigned char sM[2][SLOT];
    __shared__ int scount[2][NP], sstop[2];
    __shared__ int ndone;
    __shared__ __align__(8) uint64_t full_bar[2], empty_bar[2];

    const BlendSite site = blend_site<BATCH, 1>(bb, P, W, H);
    if (BATCH) {
        W = site.W;
        H = site.H;
        uv += site.row_off;
        conic += 3 * site.row_off;
        opacity += site.op_off;
        feature += (size_t)C * site.feat_off;
        out += (size_t)C * site.pix_off;
        final_T += site.pix_off;
        ncontrib += site.pix_off;
    }
    const int2 range = tile_range[site.tidx];
    const float bx0 = (float)(site.tx * kTile), by0 = (float)(site.ty * kTile);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        mbar_init(&full_bar[0], 32 * NP);
        mbar_init(&full_bar[1], 32 * NP);
        mbar_init(&empty_bar[0], NC);
        mbar_init(&empty_bar[1], NC);
        ndone = 0;
    }
    __syncthreads();

    if (warp >= NC) {
        // ------------------------------------------------------- producers
        // Producer warp pw gathers list positions [start + pw SUB, start +
        // (pw + 1) SUB) and compacts the kept ones, in list order, into its
        // own part [pw SUB, pw SUB + count) of the slot: the parts follow one
        // another in list order, so no prefix across producer warps is needed
        // and each round is written as soon as it is culled.
        const int pw = warp - NC;
        for (int k = 0, start = range.x;; ++k, start += SLOT) {
            const int s = k & 1;
            // One producer thread waits for the slot and decides for all
            // (so a timeout never splits the producers at their barrier).
            if (pw == 0 && lane == 0) {
                if (!mbar_wait_one(&empty_bar[s], ((k >> 1) & 1) ^ 1, wait_limit)) sstop[s] = 2;
                else sstop[s] = (start >= range.y || *(volatile int *)&ndone >= NC) ? 1 : 0;
            }
            producer_sync<NP>();
            if (sstop[s] == 2) return;  // gave up waiting: the consumers time out too
            const bool stop = sstop[s] != 0;
            int n = 0;
            if (!stop) {
                const int j0 = start + pw * SUB;
                float4 *dA = sA[s] + pw * SUB, *dB = sB[s] + pw * SUB, *dF = sF[s] + pw * SUB;
                unsigned char *dM = sM[s] + pw * SUB;
#pragma unroll 2
                for (int r = 0; r < PER; ++r) {
                    const int j = j0 + r * 32 + lane;  // list order: round, lane
                    float4 A, B, F;
                    int G;
                    unsigned M;
                    bool keep = false;
                    if (j < range.y)
                        keep = gather_entry<C, NPIX, kTile, NPB>(j, site.P, idx_sorted, uv, conic, opacity, feature, bx0,
                                                                 by0, A, B, F, G, M, EntryMasks{nullptr, emask});
                    const unsigned ballot = __ballot_sync(0xffffffffu, keep);
                    if (keep) {
                        const int pos = n + __popc(ballot & ((1u << lane) - 1u));
                        dA[pos] = A;
                        dB[pos] = B;
                        dF[pos] = F;
                        dM[pos] = (unsigned char)M;
                    }
                    n += __popc(ballot);
                }
            }
            if (lane == 0) scount[s][pw] = stop ? -1 : n;
            mbar_arrive(&full_bar[s]);  // releases this thread's slot writes
            if (stop) return;
        }
    }

    // ------------------------------------------------------------ consumers
    // (the warp blocks of blend_fwd_small_kernel: 8 columns by 4 NPIX rows)
    const int px = site.tx * kTile + 8 * (warp & 1) + (lane & 7);
    const int py0 = site.ty * kTile + 4 * NPIX * (warp >> 1) + (lane >> 3) * NPIX;
    const unsigned wbit = 1u << warp;
    const float fx = (float)px;
    float fy[NPIX], T[NPIX], F[NPIX][4];
    int last[NPIX];
    bool done[NPIX];
#pragma unroll
    for (int i = 0; i < NPIX; ++i) {
        fy[i] = (float)(py0 + i);
        T[i] = 1.0f;
        last[i] = 0;
        done[i] = !(px < W && py0 + i < H);
#pragma unroll
        for (int q = 0; q < 4; ++q) F[i][q] = 0.0f;
    }
    bool counted = false;
    for (int k = 0;; ++k) {
        const int s = k & 1;
        if (!mbar_wait_warp(&full_bar[s], (k >> 1) & 1, wait_limit)) break;
        if (scount[s][0] < 0) break;
#pragma unroll
        for (int q = 0; q < NP; ++q)
            fwd_walk_batch<C, NPIX>(scount[s][q], sA[s] + q * SUB, sB[s] + q * SUB, sF[s] + q * SUB,
                                    sM[s] + q * SUB, wbit, fx, fy, done, T, F, last, range.x);
        bool all_done = true;
#pragma unroll
        for (int i = 0; i < NPIX; ++i) all_done &= done[i];
        if (!counted && __all_sync(0xffffffffu, all_done)) {
            counted = true;
            if (lane == 0) atomicAdd(&ndone, 1);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty_bar[s]);
    }
#pragma unroll
    for (int i = 0; i < NPIX; ++i) {
        const int py = py0 + i;
        if (px < W && py < H) {
            const int pix = py * W + px;
            final_T[pix] = T[i];
            ncontrib[pix] = last[i];
#pragma unroll
            for (int q = 0; q < C; ++q) out[(size_t)q * H * W + pix] = F[i][q] + T[i] * bg;
        }
    }
}

// Reduce-scatter of N values over a warp in five halving steps.  At each
// step (partner lane ^ O) a lane group holding n slots splits them: the
// group with bit O clear keeps the first ceil(n/2), the other the rest, and
// each lane sends the half it drops, so a step costs ceil(n/2) shuffles:
// 9 values take 5 + 3 + 2 + 1 + 1 = 12 shuffles (16 when padded to a
// power of two).  Afterwards v[0] of the lane that scatter_slot<N> names
// for a slot holds that slot's warp total.
template <int N, int O>
struct ReduceScatter {
    static __device__ __forceinline__ void run(float *v, int lane) {
        constexpr int LO = (N + 1) / 2, HI = N - LO;
        const bool up = (lane & O) != 0;
#pragma unroll
        for (int k = 0; k < LO; ++k) {
            const float a = v[k];
            const float b = k < HI ? v[LO + k] : 0.0f;
            v[k] = (up ? b : a) + __shfl_xor_sync(0xffffffffu, up ? a : b, O);
        }
        ReduceScatter<LO, O / 2>::run(v, lane);
    }
};
template <int N>
struct ReduceScatter<N, 0> {
    static __device__ __forceinline__ void run(float *, int) {}
};

// The slot whose total lane `lane` holds after ReduceScatter<N, 16>, or -1.
template <int N>
__device__ __forceinline__ int scatter_slot(int lane) {
    int n = N, real = N, slot = 0;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const int lo = (n + 1) / 2;
        if (lane & o) {
            slot += lo;
            real = max(0, real - lo);
        } else {
            real = min(real, lo);
        }
        n = lo;
    }
    return real >= 1 ? slot : -1;
}

// A Gaussian's per-warp gradient goes out as direct atomics from each
// contributing lane when at most this many lanes contribute, else through a
// warp reduce-scatter first.  Same-address atomics serialise, the reduction
// costs a fixed 9-12 shuffles per value set (6 + C values): the measured
// optimum of the two at 1M Gaussians / 1080p is 12-16 lanes (with 16-shuffle
// reductions, one column per lane: blend backward 0.90 ms vs 1.00 ms with
// the reduction always and 2.98 ms with atomics always).
#ifndef MSPLAT_FEW_LANES
#define MSPLAT_FEW_LANES 12
#endif
constexpr int kFewLanes = MSPLAT_FEW_LANES;

// The backward's walk over one gathered batch (entries in reverse list
// order): each warp walks only the entries that reach its rows and precede
// its largest ncontrib (a warp-uniform bit set per 32 entries), per pixel
// undoes the transmittance, accumulates dL/dalpha from the colour
// recursion carried as two scalars, and per entry sends the moments of
// h = G dL/dalpha and the colour gradients (few lanes: direct atomics;
// otherwise a reduce-scatter and one atomic per value per warp).  Shared
// by blend_bwd_small_kernel and blend_bwd_ring_kernel.
template <int C, int NPIX, bool BG>
__device__ __forceinline__ void bwd_walk_batch(int n, const float4 *sA, const float4 *sB, const float4 *sF,
                                               const int *sG, const unsigned char *sM, unsigned wbit, int warp_last,
                                               int list0, float fx, const float (&fy)[NPIX], float (&T)[NPIX],
                                               const float (&Tf)[NPIX], float (&la)[NPIX], const float (&bgd)[NPIX],
                                               float (&ad)[NPIX], float (&lfd)[NPIX], const float (&dp)[NPIX][4],
                                               const int (&last)[NPIX], int vi, float *__restrict__ dL_duv,
                                               float *__restrict__ dL_dconic, float *__restrict__ dL_dopacity,
                                               float *__restrict__ dL_dfeature) {
    constexpr int NV = 6 + C;
    const int lane = threadIdx.x & 31;
        for (int kw = 0; kw < n; kw += 32) {
          const int kk = kw + lane;
          unsigned bits = __ballot_sync(0xffffffffu, kk < n && (sM[kk] & wbit) &&
                                                         __float_as_int(sB[kk].w) - list0 < warp_last);
          while (bits) {
            const int k = kw + __ffs(bits) - 1;
            bits &= bits - 1u;
            const float4 A = sA[k], B = sB[k];
            const int jl = __float_as_int(B.w) - list0;
            const float dx = A.x - fx;
            float dy[NPIX];
#pragma unroll
            for (int i = 0; i < NPIX; ++i) dy[i] = A.y - fy[i];
            const PixPow<NPIX> pw = blend_power_n<NPIX>(A.z, A.w, B.x, dx, dy);
            const float4 f = sF[k];
            const float fv[4] = {f.x, f.y, f.z, f.w};
            const float op = B.y;
            float v[NV];
#pragma unroll
            for (int q = 0; q < NV; ++q) v[q] = 0.0f;
            bool any = false;
#pragma unroll
            for (int i = 0; i < NPIX; ++i) {
                // Branch-free: every pixel evaluates the entry; where the
                // reference skips it (past the pixel's last contributor,
                // alpha < 1/255) the state keeps its value and the terms
                // added are zeros (measured 8 % faster than branching around).
                const float power = pw.v[i];
                const float G = __expf(power);
                const float alpha = fminf(0.99f, op * G);
                const bool ok = !(jl >= last[i] || power > 0.0f) && !(alpha < 1.0f / 255.0f);
                any |= ok;
                const float inv1m = __fdividef(1.f, 1.f - alpha);
                const float Tn = T[i] * inv1m;
                const float dcol = ok ? alpha * Tn : 0.0f;
                float fd = 0.0f;  // colour . dL/dpix
#pragma unroll
                for (int q = 0; q < C; ++q) {
                    fd += fv[q] * dp[i][q];
                    v[6 + q] += dcol * dp[i][q];
                }
                const float adn = la[i] * lfd[i] + (1.f - la[i]) * ad[i];
                float dL_dalpha = fd - adn;
                dL_dalpha *= Tn;
                if (BG) dL_dalpha += (-Tf[i] * inv1m) * bgd[i];
                // Moments of h = G dL/dalpha over the pixels; the uv, conic
                // and opacity gradients are linear in them (finished per
                // Gaussian by blend_grad_finish_kernel).
                const float h = ok ? G * dL_dalpha : 0.0f;
                const float hdx = h * dx, hdy = h * dy[i];
                v[0] += h;
                v[1] += hdx;
                v[2] += hdy;
                v[3] += hdx * dx;
                v[4] += hdx * dy[i];
                v[5] += hdy * dy[i];
                T[i] = ok ? Tn : T[i];
                ad[i] = ok ? adn : ad[i];
                lfd[i] = ok ? fd : lfd[i];
                la[i] = ok ? alpha : la[i];
            }
            const unsigned am = __ballot_sync(0xffffffffu, any);
            if (am) {
                // moments land in the gradient slots: S -> opacity, (Sx, Sy)
                // -> uv, (Sxx, Sxy, Syy) -> conic (finished per Gaussian later)
                const int g = sG[k];
                if (__popc(am) <= kFewLanes) {
                    if (any) {
                        atomicAdd(dL_dopacity + g, v[0]);
                        atomicAdd(dL_duv + 2 * g, v[1]);
                        atomicAdd(dL_duv + 2 * g + 1, v[2]);
                        atomicAdd(dL_dconic + 3 * g, v[3]);
                        atomicAdd(dL_dconic + 3 * g + 1, v[4]);
                        atomicAdd(dL_dconic + 3 * g + 2, v[5]);
#pragma unroll
                        for (int q = 0; q < C; ++q) atomicAdd(dL_dfeature + (size_t)g * C + q, v[6 + q]);
                    }
                } else {
                    ReduceScatter<NV, 16>::run(v, lane);
                    const float s = v[0];
                    if (vi >= 0) {
                        float *dst;
                        if (vi == 0) dst = dL_dopacity + g;
                        else if (vi < 3) dst = dL_duv + 2 * g + (vi - 1);
                        else if (vi < 6) dst = dL_dconic + 3 * g + (vi - 3);
                        else dst = dL_dfeature + (size_t)g * C + (vi - 6);
                        atomicAdd(dst, s);
                    }
                }
            }
          }
        }
}

// BG: the background is nonzero, so dL/dalpha has the term
// -T_final / (1 - alpha) * sum_c bg dL/dpix_c (compiled out for bg == 0).
template <int C, int NPIX, bool BG, int SPLIT, bool BATCH = false, int GE = NPIX>
__global__ void MSPLAT_BWD_BOUNDS(kTilePixels / NPIX / SPLIT)
blend_bwd_small_kernel(int P, const float2 *__restrict__ uv, const float *__restrict__ conic,
                       const float *__restrict__ opacity, const float *__restrict__ feature,
                       const int32_t *__restrict__ idx_sorted, const int2 *__restrict__ tile_range, float bg,
                       int W, int H, const float *__restrict__ final_T, const int32_t *__restrict__ ncontrib,
                       const float *__restrict__ dL_dout, float *__restrict__ dL_duv,
                       float *__restrict__ dL_dconic, float *__restrict__ dL_dopacity,
                       float *__restrict__ dL_dfeature, const unsigned char *__restrict__ emask, BlendBatch bb) {
    static_assert(!BATCH || SPLIT == 1, "batched blends render whole tiles");
    constexpr int ROWS = kTile / SPLIT, NT = kTile * ROWS / NPIX, BATCH_N = NT * GE;
    static_assert(4 * NPIX <= ROWS, "a warp block of 4 NPIX rows must fit the block's rows");
    constexpr int NV = 6 + C;
    __shared__ float4 sA[BATCH_N], sB[BATCH_N], sF[BATCH_N];
    __shared__ int sG[BATCH_N];
    __shared__ unsigned char sM[BATCH_N];
    __shared__ int scan[NT / 32];
    __shared__ int smax;
    const BlendSite site = blend_site<BATCH, SPLIT>(bb, P, W, H);
    if (BATCH) {
        W = site.W;
        H = site.H;
        uv += site.row_off;
        conic += 3 * site.row_off;
        opacity += site.op_off;
        feature += (size_t)C * site.feat_off;
        // per-camera gradient rows (opacity too: the camera's own row)
        final_T += site.pix_off;
        ncontrib += site.pix_off;
        dL_dout += (size_t)C * site.pix_off;
        dL_duv += 2 * site.row_off;
        dL_dconic += 3 * site.row_off;
        dL_dopacity += site.row_off;
        dL_dfeature += (size_t)C * site.row_off;
    }
    const int2 range = tile_range[site.tidx];
    // pixel layout, warp blocks and SPLIT as in blend_fwd_small_kernel
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row0 = site.ty * kTile + site.part * ROWS;
    const int px = site.tx * kTile + 8 * (warp & 1) + (lane & 7);
    const int py0 = row0 + 4 * NPIX * (warp >> 1) + (lane >> 3) * NPIX;
    const unsigned wbit = 1u << warp;
    const float fx = (float)px;
    const float bx0 = (float)(site.tx * kTile), by0 = (float)row0;
    const int vi = scatter_slot<NV>(lane);  // the gradient slot this lane sends after a reduction

    // Per pixel: the colour recursion of the reference (accum_rec =
    // last_alpha * last_color + (1 - last_alpha) * accum_rec per channel)
    // enters dL/dalpha only through its dot product with dL/dpix, so it is
    // carried as that scalar: ad = accum_rec . dL/dpix and lfd = last_color
    // . dL/dpix.
    float fy[NPIX], T[NPIX], Tf[NPIX], la[NPIX], bgd[NPIX], ad[NPIX], lfd[NPIX];
    float dp[NPIX][4];
    int last[NPIX];
    int mylast = 0;
#pragma unroll
    for (int i = 0; i < NPIX; ++i) {
        const int py = py0 + i;
        const bool in = px < W && py < H;
        const int pix = py * W + px;
        fy[i] = (float)py;
        Tf[i] = in ? final_T[pix] : 0.0f;
        T[i] = Tf[i];
        last[i] = in ? ncontrib[pix] : 0;
        mylast = max(mylast, last[i]);
        la[i] = 0.0f;
        bgd[i] = 0.0f;
        ad[i] = 0.0f;
        lfd[i] = 0.0f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            dp[i][q] = (in && q < C) ? dL_dout[(size_t)q * H * W + pix] : 0.0f;
            if (q < C) bgd[i] += bg * dp[i][q];
        }
    }
    if (threadIdx.x == 0) smax = 0;
    __syncthreads();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mylast = max(mylast, __shfl_xor_sync(0xffffffffu, mylast, o));
    if (lane == 0) atomicMax(&smax, mylast);
    __syncthreads();
    const int end = range.x + min(smax, range.y - range.x);
    // Entries at or past this warp's largest ncontrib touch none of its pixels.
    const int warp_last = mylast;

    for (int bend = end; bend > range.x; bend -= BATCH_N) {
        const int bstart = max(range.x, bend - BATCH_N);
        const int n = gather_small<C, NPIX, true, ROWS, GE>(bend - 1, -1, bstart, bend, site.P, idx_sorted, uv, conic,
                                                        opacity, feature, bx0, by0, sA, sB, sF, sG, sM, scan,
                                                        false, EntryMasks{emask, nullptr});
        bwd_walk_batch<C, NPIX, BG>(n, sA, sB, sF, sG, sM, wbit, warp_last, range.x, fx, fy, T, Tf, la, bgd, ad,
                                    lfd, dp, last, vi, dL_duv, dL_dconic, dL_dopacity, dL_dfeature);
        // no barrier here: the next gather's first barrier orders the batches
    }
}

// ===================================================================
// Backward blend as a producer / consumer ring (C <= 4): NP producer warps
// gather, cull and mask each 256-entry batch of a tile's list from its end
// (the same per-entry work as gather_small with dir = -1), each compacting
// its share, in reverse list order, into its own part of one of two
// shared-memory slots; the consumer warps (NPIX pixels per thread, the
// warp blocks of blend_bwd_small_kernel) walk the other slot part by part
// with the same code (bwd_walk_batch).  Hand-off and bounded waits as in
// blend_fwd_ring_kernel: per slot a "full" mbarrier (every producer thread
// arrives after its writes) and an "empty" one (each consumer warp
// arrives); the number of batches follows from the block's largest
// ncontrib, known to all before the first.  Results equal
// blend_bwd_small_kernel's up to the order of the gradient atomics (the
// same entries reach each warp in the same order with the same per-pair
// code).
// ===================================================================
template <int C, int NPIX, int NP, bool BG, bool BATCH = false>
__global__ void MSPLAT_RING_BOUNDS(kTilePixels / NPIX + 32 * NP)
blend_bwd_ring_kernel(int P, const float2 *__restrict__ uv, const float *__restrict__ conic,
                      const float *__restrict__ opacity, const float *__restrict__ feature,
                      const int32_t *__restrict__ idx_sorted, const int2 *__restrict__ tile_range, float bg, int W,
                      int H, const float *__restrict__ final_T, const int32_t *__restrict__ ncontrib,
                      const float *__restrict__ dL_dout, float *__restrict__ dL_duv, float *__restrict__ dL_dconic,
                      float *__restrict__ dL_dopacity, float *__restrict__ dL_dfeature,
                      const unsigned char *__restrict__ emask, BlendBatch bb, int wait_limit) {
    constexpr int NT = kTilePixels / NPIX;  // consumer threads
    constexpr int NCW = NT / 32;            // consumer warps
    constexpr int SLOT = 256;               // entries per batch
    constexpr int SUB = SLOT / NP;          // entries per producer warp (its own part of the slot)
    constexpr int PER = SUB / 32;           // gather rounds per producer warp
    constexpr int NV = 6 + C;
    static_assert(SLOT % (32 * NP) == 0, "producer warps must split a batch evenly");
    __shared__ float4 sA[2][SLOT], sB[2][SLOT], sF[2][SLOT];
    __shared__ int sG[2][SLOT];
    __shared__ unsigned char sM[2][SLOT];
    __shared__ int scount[2][NP], sstop[2];
    __shared__ int smax;
    __shared__ __align__(8) uint64_t full_bar[2], empty_bar[2];

    const BlendSite site = blend_site<BATCH, 1>(bb, P, W, H);
    if (BATCH) {
        W = site.W;
        H = site.H;
        uv += site.row_off;
        conic += 3 * site.row_off;
        opacity += site.op_off;
        feature += (size_t)C * site.feat_off;
        final_T += site.pix_off;
        ncontrib += site.pix_off;
        dL_dout += (size_t)C * site.pix_off;
        dL_duv += 2 * site.row_off;
        dL_dconic += 3 * site.row_off;
        dL_dopacity += site.row_off;
        dL_dfeature += (size_t)C * site.row_off;
    }
    const int2 range = tile_range[site.tidx];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool consumer = warp < NCW;
    const float bx0 = (float)(site.tx * kTile), by0 = (float)(site.ty * kTile);
    if (threadIdx.x == 0) {
        smax = 0;
        mbar_init(&full_bar[0], 32 * NP);
        mbar_init(&full_bar[1], 32 * NP);
        mbar_init(&empty_bar[0], NCW);
        mbar_init(&empty_bar[1], NCW);
    }
    __syncthreads();

    // consumer pixels and state (as blend_bwd_small_kernel)
    const int px = site.tx * kTile + 8 * (warp & 1) + (lane & 7);
    const int py0 = site.ty * kTile + 4 * NPIX * (warp >> 1) + (lane >> 3) * NPIX;
    float fy[NPIX], T[NPIX], Tf[NPIX], la[NPIX], bgd[NPIX], ad[NPIX], lfd[NPIX];
    float dp[NPIX][4];
    int last[NPIX];
    int mylast = 0;
    if (consumer) {
#pragma unroll
        for (int i = 0; i < NPIX; ++i) {
            const int py = py0 + i;
            const bool in = px < W && py < H;
            const int pix = py * W + px;
            fy[i] = (float)py;
            Tf[i] = in ? final_T[pix] : 0.0f;
            T[i] = Tf[i];
            last[i] = in ? ncontrib[pix] : 0;
            mylast = max(mylast, last[i]);
            la[i] = 0.0f;
            bgd[i] = 0.0f;
            ad[i] = 0.0f;
            lfd[i] = 0.0f;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                dp[i][q] = (in && q < C) ? dL_dout[(size_t)q * H * W + pix] : 0.0f;
                if (q < C) bgd[i] += bg * dp[i][q];
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mylast = max(mylast, __shfl_xor_sync(0xffffffffu, mylast, o));
        if (lane == 0) atomicMax(&smax, mylast);
    }
    __syncthreads();
    const int end = range.x + min(smax, range.y - range.x);
    const int nb = end > range.x ? (end - range.x + SLOT - 1) / SLOT : 0;

    if (!consumer) {
        // ------------------------------------------------------- producers
        const int pw = warp - NCW;
        for (int k = 0; k < nb; ++k) {
            const int s = k & 1;
            if (pw == 0 && lane == 0) sstop[s] = mbar_wait_one(&empty_bar[s], ((k >> 1) & 1) ^ 1, wait_limit) ? 0 : 2;
            producer_sync<NP>();
            if (sstop[s] == 2) return;  // gave up waiting: the consumers time out too
            const int bend = end - k * SLOT, bstart = max(range.x, bend - SLOT);
            float4 *dA = sA[s] + pw * SUB, *dB = sB[s] + pw * SUB, *dF = sF[s] + pw * SUB;
            int *dG = sG[s] + pw * SUB;
            unsigned char *dM = sM[s] + pw * SUB;
            int n = 0;
#pragma unroll 2
            for (int r = 0; r < PER; ++r) {
                const int j = bend - 1 - (pw * SUB + r * 32 + lane);  // reverse list order: part, round, lane
                float4 A, B, F;
                int G;
                unsigned M;
                bool keep = false;
                if (j >= bstart)
                    keep = gather_entry<C, NPIX, kTile>(j, site.P, idx_sorted, uv, conic, opacity, feature, bx0, by0,
                                                        A, B, F, G, M, EntryMasks{emask, nullptr});
                const unsigned ballot = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    const int pos = n + __popc(ballot & ((1u << lane) - 1u));
                    dA[pos] = A;
                    dB[pos] = B;
                    dF[pos] = F;
                    dG[pos] = G;
                    dM[pos] = (unsigned char)M;
                }
                n += __popc(ballot);
            }
            if (lane == 0) scount[s][pw] = n;
            mbar_arrive(&full_bar[s]);  // releases this thread's slot writes
        }
        return;
    }

    // ------------------------------------------------------------ consumers
    const unsigned wbit = 1u << warp;
    const float fx = (float)px;
    const int vi = scatter_slot<NV>(lane);
    for (int k = 0; k < nb; ++k) {
        const int s = k & 1;
        if (!mbar_wait_warp(&full_bar[s], (k >> 1) & 1, wait_limit)) break;
#pragma unroll
        for (int q = 0; q < NP; ++q)
            bwd_walk_batch<C, NPIX, BG>(scount[s][q], sA[s] + q * SUB, sB[s] + q * SUB, sF[s] + q * SUB,
                                        sG[s] + q * SUB, sM[s] + q * SUB, wbit, mylast, range.x, fx, fy, T, Tf, la,
                                        bgd, ad, lfd, dp, last, vi, dL_duv, dL_dconic, dL_dopacity, dL_dfeature);
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty_bar[s]);
    }
}

// Turns the moments accumulated by blend_bwd_small_kernel into gradients,
// in place: with h = G dL/dalpha summed over pixels,
//   dL/dopacity = S,  dL/du = -o (a Sx + b Sy),  dL/dv = -o (c Sy + b Sx),
//   dL/dconic = (-o Sxx / 2, -o Sxy, -o Syy / 2)
// which is the reference's per-pair formula (alpha_blending.cu:231-243)
// summed: dL/dG = o dL/dalpha and dG/d(dx) = -G (a dx + b dy), etc.
__global__ void __launch_bounds__(256)
blend_grad_finish_kernel(int P, const float *__restrict__ conic, const float *__restrict__ opacity,
                         float *__restrict__ dL_duv, float *__restrict__ dL_dconic) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= P) return;
    const float o = opacity[g];
    const float a = conic[3 * g], b = conic[3 * g + 1], c = conic[3 * g + 2];
    const float sx = dL_duv[2 * g], sy = dL_duv[2 * g + 1];
    const float sxx = dL_dconic[3 * g], sxy = dL_dconic[3 * g + 1], syy = dL_dconic[3 * g + 2];
    dL_duv[2 * g] = -o * (a * sx + b * sy);
    dL_duv[2 * g + 1] = -o * (c * sy + b * sx);
    dL_dconic[3 * g] = -0.5f * o * sxx;
    dL_dconic[3 * g + 1] = -o * sxy;
    dL_dconic[3 * g + 2] = -0.5f * o * syy;
}

// blend_grad_finish_kernel over the stacked rows of a batch: row r is
// Gaussian r - row_off of its camera, whose opacity is opacity[op_off + g].
__global__ void __launch_bounds__(256)
batch_blend_grad_finish_kernel(BatchPlanView pv, int64_t rows, const float *__restrict__ conic,
                               const float *__restrict__ opacity, float *__restrict__ dL_duv,
                               float *__restrict__ dL_dconic) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    int lo = 0, hi = pv.B - 1;  // the camera of row r: last b with row_off <= r
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pv.cams[mid].row_off <= r) lo = mid;
        else hi = mid - 1;
    }
    const BatchCam &c = pv.cams[lo];
    const float o = opacity[c.op_off + (r - c.row_off)];
    const float a = conic[3 * r], b = conic[3 * r + 1], cc = conic[3 * r + 2];
    const float sx = dL_duv[2 * r], sy = dL_duv[2 * r + 1];
    const float sxx = dL_dconic[3 * r], sxy = dL_dconic[3 * r + 1], syy = dL_dconic[3 * r + 2];
    dL_duv[2 * r] = -o * (a * sx + b * sy);
    dL_duv[2 * r + 1] = -o * (cc * sy + b * sx);
    dL_dconic[3 * r] = -0.5f * o * sxx;
    dL_dconic[3 * r + 1] = -o * sxy;
    dL_dconic[3 * r + 2] = -0.5f * o * syy;
}

// Pixels per thread of the C <= 4 kernels (compile-time tunables).
#ifndef MSPLAT_BLEND_NPIX_FWD
#define MSPLAT_BLEND_NPIX_FWD 1
#endif
#ifndef MSPLAT_BLEND_NPIX_BWD
#define MSPLAT_BLEND_NPIX_BWD 2
#endif
constexpr int kBlendNpixFwd = MSPLAT_BLEND_NPIX_FWD;
constexpr int kBlendNpixBwd = MSPLAT_BLEND_NPIX_BWD;
// Entries gathered per thread per shared-memory batch (so Gaussians per
// batch = threads x this; compile-time tunables, default one per pixel).
#ifndef MSPLAT_BLEND_GATHER_FWD
#define MSPLAT_BLEND_GATHER_FWD MSPLAT_BLEND_NPIX_FWD
#endif
#ifndef MSPLAT_BLEND_GATHER_BWD
#define MSPLAT_BLEND_GATHER_BWD MSPLAT_BLEND_NPIX_BWD
#endif
constexpr int kGatherFwd = MSPLAT_BLEND_GATHER_FWD, kGatherBwd = MSPLAT_BLEND_GATHER_BWD;
// The same shape parameters for the multi-camera blend grid, tuned on the
// multi-camera workload (default: the single-camera values).
#ifndef MSPLAT_BATCH_BLEND_NPIX_FWD
#define MSPLAT_BATCH_BLEND_NPIX_FWD MSPLAT_BLEND_NPIX_FWD
#endif
#ifndef MSPLAT_BATCH_BLEND_NPIX_BWD
#define MSPLAT_BATCH_BLEND_NPIX_BWD MSPLAT_BLEND_NPIX_BWD
#endif
#ifndef MSPLAT_BATCH_BLEND_GATHER_FWD
#define MSPLAT_BATCH_BLEND_GATHER_FWD MSPLAT_BATCH_BLEND_NPIX_FWD
#endif
#ifndef MSPLAT_BATCH_BLEND_GATHER_BWD
#define MSPLAT_BATCH_BLEND_GATHER_BWD MSPLAT_BATCH_BLEND_NPIX_BWD
#endif
constexpr int kBatchNpixFwd = MSPLAT_BATCH_BLEND_NPIX_FWD, kBatchNpixBwd = MSPLAT_BATCH_BLEND_NPIX_BWD;
// The C <= 4 forward as a producer / consumer ring (blend_fwd_ring_kernel)
// with this many producer warps (2 or 4), or the gather-barrier kernel (0);
// the default is a tunable, msplat_set_blend_ring changes it at run time.
#ifndef MSPLAT_BLEND_RING_FWD
#define MSPLAT_BLEND_RING_FWD 0
#endif
#ifndef MSPLAT_BATCH_BLEND_RING_FWD
#define MSPLAT_BATCH_BLEND_RING_FWD MSPLAT_BLEND_RING_FWD
#endif
static int g_fwd_ring = MSPLAT_BLEND_RING_FWD;
static int g_batch_fwd_ring = MSPLAT_BATCH_BLEND_RING_FWD;
// The backward as a ring with 1 or 2 producer warps (0: block-barrier
// kernel); tunable default, msplat_set_blend_ring_bwd at run time.
#ifndef MSPLAT_BLEND_RING_BWD
#define MSPLAT_BLEND_RING_BWD 0
#endif
#ifndef MSPLAT_BATCH_BLEND_RING_BWD
#define MSPLAT_BATCH_BLEND_RING_BWD MSPLAT_BLEND_RING_BWD
#endif
static int g_bwd_ring = MSPLAT_BLEND_RING_BWD;
static int g_batch_bwd_ring = MSPLAT_BATCH_BLEND_RING_BWD;
// Single-camera images below this many tiles keep the barrier backward:
// with a few hundred tiles of long lists (less than one wave of blocks) the
// ring's single producer warp falls behind (256 x 256: 2.12 vs 1.96 ms;
// from 512 x 512 up the ring is as fast or faster).
constexpr int kBwdRingMinTiles = 1024;
// The forward ring takes the tuned pixels per thread (MSPLAT_BLEND_NPIX_FWD)
// on single-camera images of at least this many tiles and one pixel per
// thread below: two pixels per thread halve the per-entry overhead but
// coarsen the warp blocks (8 x 8 pixels instead of 8 x 4), which pays where
// Gaussians cover many pixels (1920 x 1080: 0.265 -> 0.237 ms) and not on
// smaller images of the same scene (1280 x 720: 0.199 -> 0.220 ms; 512 x
// 512: 0.429 -> 0.548 ms).
constexpr int kFwdRingWideMinTiles = 6000;
constexpr int kBatchGatherFwd = MSPLAT_BATCH_BLEND_GATHER_FWD, kBatchGatherBwd = MSPLAT_BATCH_BLEND_GATHER_BWD;
// Blocks per tile of the C <= 4 kernels (1 or 2: whole tiles, or halves of
// 8 rows with their own gather, cull and end; compile-time tunables).
#ifndef MSPLAT_BLEND_SPLIT_FWD
#define MSPLAT_BLEND_SPLIT_FWD 1
#endif
#ifndef MSPLAT_BLEND_SPLIT_BWD
#define MSPLAT_BLEND_SPLIT_BWD 1
#endif
constexpr int kSplitFwd = MSPLAT_BLEND_SPLIT_FWD, kSplitBwd = MSPLAT_BLEND_SPLIT_BWD;
// The forward's entry masks carry over to the backward when both render whole tiles.
constexpr bool kEntryMasks = kSplitFwd == 1 && kSplitBwd == 1;


// The forward for C > 4: one walk over the list when the channels fit 64
// (the smallest of 16 / 32 / 40 / 64 that holds them), else walks of 32
// channels.  Every channel's colour is the same sum either way.
template <bool BATCH>
inline void launch_fwd_general(int C, dim3 grid, cudaStream_t stream, int P, const float2 *uv, const float *conic,
                               const float *opacity, const float *feature, const int32_t *idx, const int2 *tr,
                               float bg, int W, int H, float *out, float *final_T, int32_t *nc,
                               const BlendBatch &bb) {
#define MSPLAT_FWDG(CM, C0)                                                                                      \
    do {                                                                                                         \
        const size_t smem = (size_t)CM * kBatch * sizeof(float);                                                 \
        cudaFuncSetAttribute(blend_fwd_kernel<CM, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        launch(blend_fwd_kernel<CM, BATCH>, grid, kBlendThreads, smem, stream, P, C, C0, uv, conic, opacity,       \
               feature, idx, tr, bg, W, H, out, final_T, nc, bb);                                                \
    } while (0)
    if (C <= 16) MSPLAT_FWDG(16, 0);
    else if (C <= 32) MSPLAT_FWDG(32, 0);
    else if (C <= 40) MSPLAT_FWDG(40, 0);
    else if (C <= 64) MSPLAT_FWDG(64, 0);
    else
        for (int c0 = 0; c0 < C; c0 += 32) {
            if (C - c0 <= 4) MSPLAT_FWDG(4, c0);
            else if (C - c0 <= 16) MSPLAT_FWDG(16, c0);
            else MSPLAT_FWDG(32, c0);
        }
#undef MSPLAT_FWDG
}

// The one-walk backward for 4 < C <= 64 (blend_bwd_wide_kernel): the
// smallest channel capacity that holds C.
template <bool BATCH>
inline void launch_bwd_wide(int C, dim3 grid, cudaStream_t stream, int P, const float2 *uv, const float *conic,
                            const float *opacity, const float *feature, const int32_t *idx, const int2 *tr, float bg,
                            int W, int H, const float *fT, const int32_t *nci, const float *dout, float *duv,
                            float *dcon, float *dop, float *dfeat, const BlendBatch &bb) {
#define MSPLAT_WIDE(CM)                                                                                          \
    do {                                                                                                         \
        const size_t smem = blend_bwd_wide_smem<CM>();                                                           \
        cudaFuncSetAttribute(blend_bwd_wide_kernel<CM, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,       \
                             (int)smem);                                                                         \
        launch(blend_bwd_wide_kernel<CM, BATCH>, grid, kBlendThreads, smem, stream, P, C, uv, conic, opacity,      \
               feature, idx, tr, bg, W, H, fT, nci, dout, duv, dcon, dop, dfeat, bb);                            \
    } while (0)
    if (C <= 16) MSPLAT_WIDE(16);
    else if (C <= 32) MSPLAT_WIDE(32);
    else if (C <= 40) MSPLAT_WIDE(40);
    else MSPLAT_WIDE(64);
#undef MSPLAT_WIDE
}
constexpr int kWideMaxC = 64;  // channels of the one-walk backward; more go through chunked walks

template <int C>
void launch_small(bool bwd, dim3 grid, cudaStream_t stream, int P, const float2 *uv, const float *conic,
                  const float *opacity, const float *feature, const int32_t *idx, const int2 *tr, float bg, int W,
                  int H, float *out, float *final_T, int32_t *nc, const float *fT, const int32_t *nci,
                  const float *dout, float *duv, float *dcon, float *dop, float *dfeat, unsigned char *emask) {
    const dim3 gf(grid.x, grid.y * kSplitFwd), gb(grid.x, grid.y * kSplitBwd);
    if (!kEntryMasks) emask = nullptr;
    constexpr int tf = kTilePixels / kBlendNpixFwd / kSplitFwd, tb = kTilePixels / kBlendNpixBwd / kSplitBwd;
    if (!bwd && (g_fwd_ring == 2 || g_fwd_ring == 4)) {
        // the tuned pixels per thread on images of at least kFwdRingWideMinTiles tiles, one below
        const bool wide = (int)(grid.x * grid.y) >= kFwdRingWideMinTiles;
#define MSPLAT_FWD_RING(NP, NPX)                                                                                 \
    launch(blend_fwd_ring_kernel<C, NP, false, NPX, kBlendNpixBwd>, grid, kTilePixels / NPX + 32 * NP, 0, stream, P, \
           uv, conic, opacity, feature, idx, tr, bg, W, H, out, final_T, nc, emask, BlendBatch{}, g_wait_limit)
        if (g_fwd_ring == 2 && wide) MSPLAT_FWD_RING(2, kBlendNpixFwd);
        else if (g_fwd_ring == 2) MSPLAT_FWD_RING(2, 1);
        else if (wide) MSPLAT_FWD_RING(4, kBlendNpixFwd);
        else MSPLAT_FWD_RING(4, 1);
#undef MSPLAT_FWD_RING
    } else if (!bwd)
        launch(blend_fwd_small_kernel<C, kBlendNpixFwd, kSplitFwd, false, kGatherFwd, kBlendNpixBwd>, gf, tf, 0, stream,
            P, uv, conic, opacity, feature, idx, tr, bg, W, H, out, final_T, nc, emask, BlendBatch{});
    else if ((g_bwd_ring == 1 || g_bwd_ring == 2) && (int)(grid.x * grid.y) >= kBwdRingMinTiles) {
        constexpr int tr0 = kTilePixels / kBlendNpixBwd;
#define MSPLAT_BWD_RING(NP, BGV)                                                                                 \
    launch(blend_bwd_ring_kernel<C, kBlendNpixBwd, NP, BGV>, grid, tr0 + 32 * NP, 0, stream, P, uv, conic, opacity, \
           feature, idx, tr, bg, W, H, fT, nci, dout, duv, dcon, dop, dfeat, emask, BlendBatch{}, g_wait_limit)
        if (g_bwd_ring == 1 && bg != 0.0f) MSPLAT_BWD_RING(1, true);
        else if (g_bwd_ring == 1) MSPLAT_BWD_RING(1, false);
        else if (bg != 0.0f) MSPLAT_BWD_RING(2, true);
        else MSPLAT_BWD_RING(2, false);
#undef MSPLAT_BWD_RING
    } else if (bg != 0.0f)
        launch(blend_bwd_small_kernel<C, kBlendNpixBwd, true, kSplitBwd, false, kGatherBwd>, gb, tb, 0, stream,
            P, uv, conic, opacity, feature, idx, tr, bg, W, H, fT, nci, dout, duv, dcon, dop, dfeat, emask,
            BlendBatch{});
    else
        launch(blend_bwd_small_kernel<C, kBlendNpixBwd, false, kSplitBwd, false, kGatherBwd>, gb, tb, 0, stream,
            P, uv, conic, opacity, feature, idx, tr, bg, W, H, fT, nci, dout, duv, dcon, dop, dfeat, emask,
            BlendBatch{});
}

inline void dispatch_small(bool bwd, int C, dim3 grid, cudaStream_t stream, int P, const float2 *uv,
                           const float *conic, const float *opacity, const float *feature, const int32_t *idx,
                           const int2 *tr, float bg, int W, int H, float *out, float *final_T, int32_t *nc,
                           const float *fT, const int32_t *nci, const float *dout, float *duv, float *dcon,
                           float *dop, float *dfeat, unsigned char *emask) {
    switch (C) {
#define MSPLAT_SMALL(CC)                                                                                       \
    case CC:                                                                                                   \
        launch_small<CC>(bwd, grid, stream, P, uv, conic, opacity, feature, idx, tr, bg, W, H, out, final_T,   \
                         nc, fT, nci, dout, duv, dcon, dop, dfeat, emask);                                    \
        break;
        MSPLAT_SMALL(1) MSPLAT_SMALL(2) MSPLAT_SMALL(3) MSPLAT_SMALL(4)
#undef MSPLAT_SMALL
        default: break;
    }
}

}  // namespace msplat

using namespace msplat;

static int blend_forward(int P, int C, const float *uv, const float *conic, const float *opacity, const float *feature,
                         const int32_t *idx_sorted, const int32_t *tile_range, float bg, int W, int H, float *out,
                         float *final_T, int32_t *ncontrib, unsigned char *entry_masks, cudaStream_t stream) {
    if (P < 0 || C <= 0 || W <= 0 || H <= 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "alpha_blending_forward: bad sizes P=%d C=%d W=%d H=%d",
                         P, C, W, H);
    if (!tile_range || !out || !final_T || !ncontrib || (P > 0 && (!uv || !conic || !opacity || !feature)))
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "alpha_blending_forward: null pointer");
    const dim3 grid(ceil_div(W, kTile), ceil_div(H, kTile));
    if (C <= 4) {
        dispatch_small(false, C, grid, stream, P, (const float2 *)uv, conic, opacity, feature, idx_sorted,
                       (const int2 *)tile_range, bg, W, H, out, final_T, ncontrib, nullptr, nullptr, nullptr,
                       nullptr, nullptr, nullptr, nullptr, entry_masks);
        return check_launch("alpha_blending_forward");
    }
    // one walk for up to 64 channels, chunks of 32 beyond
    launch_fwd_general<false>(C, grid, stream, P, (const float2 *)uv, conic, opacity, feature, idx_sorted,
                              (const int2 *)tile_range, bg, W, H, out, final_T, ncontrib, BlendBatch{});
    return check_launch("alpha_blending_forward");
}

static int blend_backward(int P, int C, const float *uv, const float *conic, const float *opacity,
                          const float *feature, const int32_t *idx_sorted, const int32_t *tile_range, float bg, int W,
                          int H, const float *final_T, const int32_t *ncontrib, const float *dL_dout, float *dL_duv,
                          float *dL_dconic, float *dL_dopacity, float *dL_dfeature, const unsigned char *entry_masks,
                          cudaStream_t stream) {
    if (P < 0 || C <= 0 || W <= 0 || H <= 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "alpha_blending_backward: bad sizes");
    if (!tile_range || !final_T || !ncontrib || !dL_dout ||
        (P > 0 && (!uv || !conic || !opacity || !feature || !dL_duv || !dL_dconic || !dL_dopacity || !dL_dfeature)))
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "alpha_blending_backward: null pointer");
    if (P == 0) return MSPLAT_OK;
    const dim3 grid(ceil_div(W, kTile), ceil_div(H, kTile));
    if (C <= 4) {
        dispatch_small(true, C, grid, stream, P, (const float2 *)uv, conic, opacity, feature, idx_sorted,
                       (const int2 *)tile_range, bg, W, H, nullptr, nullptr, nullptr, final_T, ncontrib, dL_dout,
                       dL_duv, dL_dconic, dL_dopacity, dL_dfeature, const_cast<unsigned char *>(entry_masks));
        launch(blend_grad_finish_kernel, ceil_div(P, 256), 256, 0, stream, P, conic, opacity, dL_duv, dL_dconic);
        return check_launch("alpha_blending_backward");
    }
    if (C <= kWideMaxC) {
        launch_bwd_wide<false>(C, grid, stream, P, (const float2 *)uv, conic, opacity, feature, idx_sorted,
                               (const int2 *)tile_range, bg, W, H, final_T, ncontrib, dL_dout, dL_duv, dL_dconic,
                               dL_dopacity, dL_dfeature, BlendBatch{});
        return check_launch("alpha_blending_backward");
    }
    for (int c0 = 0; c0 < C; c0 += kBwdC)
        launch(blend_bwd_kernel<false>, grid, kBlendThreads, 0, stream, P, C, c0, (const float2 *)uv, conic, opacity, feature,
                                                             idx_sorted, (const int2 *)tile_range, bg, W, H, final_T,
                                                             ncontrib, dL_dout, dL_duv, dL_dconic, dL_dopacity,
                                                             dL_dfeature, BlendBatch{});
    return check_launch("alpha_blending_backward");
}

extern "C" int msplat_alpha_blending_forward(int P, int C, const float *uv, const float *conic,
                                             const float *opacity, const float *feature,
                                             const int32_t *idx_sorted, const int32_t *tile_range,
                                             float bg, int W, int H, float *out, float *final_T,
                                             int32_t *ncontrib, msplat_stream_t stream) {
    return blend_forward(P, C, uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, out, final_T, ncontrib,
                         nullptr, stream);
}

extern "C" int msplat_alpha_blending_forward_masks(int P, int C, const float *uv, const float *conic,
                                                   const float *opacity, const float *feature,
                                                   const int32_t *idx_sorted, const int32_t *tile_range, float bg,
                                                   int W, int H, float *out, float *final_T, int32_t *ncontrib,
                                                   unsigned char *entry_masks, msplat_stream_t stream) {
    return blend_forward(P, C, uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, out, final_T, ncontrib,
                         entry_masks, stream);
}

extern "C" int msplat_alpha_blending_backward(int P, int C, const float *uv, const float *conic,
                                              const float *opacity, const float *feature,
                                              const int32_t *idx_sorted, const int32_t *tile_range,
                                              float bg, int W, int H, const float *final_T,
                                              const int32_t *ncontrib, const float *dL_dout,
                                              float *dL_duv, float *dL_dconic, float *dL_dopacity,
                                              float *dL_dfeature, msplat_stream_t stream) {
    return blend_backward(P, C, uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, final_T, ncontrib,
                          dL_dout, dL_duv, dL_dconic, dL_dopacity, dL_dfeature, nullptr, stream);
}

extern "C" int msplat_alpha_blending_backward_masks(int P, int C, const float *uv, const float *conic,
                                                    const float *opacity, const float *feature,
                                                    const int32_t *idx_sorted, const int32_t *tile_range, float bg,
                                                    int W, int H, const float *final_T, const int32_t *ncontrib,
                                                    const float *dL_dout, float *dL_duv, float *dL_dconic,
                                                    float *dL_dopacity, float *dL_dfeature,
                                                    const unsigned char *entry_masks, msplat_stream_t stream) {
    return blend_backward(P, C, uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, final_T, ncontrib,
                          dL_dout, dL_duv, dL_dconic, dL_dopacity, dL_dfeature, entry_masks, stream);
}

// ------------------------------------------------------------ batches
namespace {

template <int C>
void launch_small_batch(bool bwd, int tiles, cudaStream_t stream, const BlendBatch &bb, const float2 *uv,
                        const float *conic, const float *opacity, const float *feature, const int32_t *idx,
                        const int2 *tr, float bg, float *out, float *final_T, int32_t *nc, const float *fT,
                        const int32_t *nci, const float *dout, float *duv, float *dcon, float *dop, float *dfeat,
                        unsigned char *emask) {
    constexpr int tf = kTilePixels / kBatchNpixFwd, tb = kTilePixels / kBatchNpixBwd;
    if (!bwd && g_batch_fwd_ring == 2)
        launch(blend_fwd_ring_kernel<C, 2, true, kBatchNpixFwd, kBatchNpixBwd>, tiles, kTilePixels / kBatchNpixFwd + 64, 0, stream, 0, uv, conic, opacity, feature,
               idx, tr, bg, 1, 1, out, final_T, nc, emask, bb, g_wait_limit);
    else if (!bwd && g_batch_fwd_ring == 4)
        launch(blend_fwd_ring_kernel<C, 4, true, kBatchNpixFwd, kBatchNpixBwd>, tiles, kTilePixels / kBatchNpixFwd + 128, 0, stream, 0, uv, conic, opacity,
               feature, idx, tr, bg, 1, 1, out, final_T, nc, emask, bb, g_wait_limit);
    else if (!bwd)
        launch(blend_fwd_small_kernel<C, kBatchNpixFwd, 1, true, kBatchGatherFwd, kBatchNpixBwd>, tiles, tf, 0,
               stream, 0, uv, conic, opacity, feature, idx, tr, bg, 1, 1, out, final_T, nc, emask, bb);
    else if (g_batch_bwd_ring == 1 || g_batch_bwd_ring == 2) {
#define MSPLAT_BWD_RING(NP, BGV)                                                                                  \
    launch(blend_bwd_ring_kernel<C, kBatchNpixBwd, NP, BGV, true>, tiles, tb + 32 * NP, 0, stream, 0, uv, conic,     \
           opacity, feature, idx, tr, bg, 1, 1, fT, nci, dout, duv, dcon, dop, dfeat, emask, bb, g_wait_limit)
        if (g_batch_bwd_ring == 1 && bg != 0.0f) MSPLAT_BWD_RING(1, true);
        else if (g_batch_bwd_ring == 1) MSPLAT_BWD_RING(1, false);
        else if (bg != 0.0f) MSPLAT_BWD_RING(2, true);
        else MSPLAT_BWD_RING(2, false);
#undef MSPLAT_BWD_RING
    } else if (bg != 0.0f)
        launch(blend_bwd_small_kernel<C, kBatchNpixBwd, true, 1, true, kBatchGatherBwd>, tiles, tb, 0, stream, 0, uv,
               conic, opacity, feature, idx, tr, bg, 1, 1, fT, nci, dout, duv, dcon, dop, dfeat, emask, bb);
    else
        launch(blend_bwd_small_kernel<C, kBatchNpixBwd, false, 1, true, kBatchGatherBwd>, tiles, tb, 0, stream, 0,
               uv, conic, opacity, feature, idx, tr, bg, 1, 1, fT, nci, dout, duv, dcon, dop, dfeat, emask, bb);
}

void dispatch_small_batch(bool bwd, int C, int tiles, cudaStream_t stream, const BlendBatch &bb, const float2 *uv,
                          const float *conic, const float *opacity, const float *feature, const int32_t *idx,
                          const int2 *tr, float bg, float *out, float *final_T, int32_t *nc, const float *fT,
                          const int32_t *nci, const float *dout, float *duv, float *dcon, float *dop, float *dfeat,
                          unsigned char *emask) {
    switch (C) {
#define MSPLAT_SMALL_B(CC)                                                                                   \
    case CC:                                                                                                 \
        launch_small_batch<CC>(bwd, tiles, stream, bb, uv, conic, opacity, feature, idx, tr, bg, out, final_T, \
                               nc, fT, nci, dout, duv, dcon, dop, dfeat, emask);                             \
        break;
        MSPLAT_SMALL_B(1) MSPLAT_SMALL_B(2) MSPLAT_SMALL_B(3) MSPLAT_SMALL_B(4)
#undef MSPLAT_SMALL_B
        default: break;
    }
}

}  // namespace

static int batch_blend_forward(const void *plan, int B, int total_tiles, int C, int feature_per_camera,
                               const float *uv, const float *conic, const float *opacity, const float *feature,
                               const int32_t *idx_sorted, const int32_t *tile_range, float bg, float *out,
                               float *final_T, int32_t *ncontrib, unsigned char *entry_masks, cudaStream_t stream) {
    if (B <= 0 || total_tiles < 0 || C <= 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_alpha_blending_forward: bad sizes B=%d C=%d", B, C);
    if (!plan || !uv || !conic || !opacity || !feature || !tile_range || !out || !final_T || !ncontrib)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_alpha_blending_forward: null pointer");
    if (total_tiles == 0) return MSPLAT_OK;
    const BlendBatch bb{batch_plan_view(plan, B), feature_per_camera};
    if (C <= 4) {
        dispatch_small_batch(false, C, total_tiles, stream, bb, (const float2 *)uv, conic, opacity, feature, idx_sorted,
                             (const int2 *)tile_range, bg, out, final_T, ncontrib, nullptr, nullptr, nullptr, nullptr,
                             nullptr, nullptr, nullptr, entry_masks);
        return check_launch("batch_alpha_blending_forward");
    }
    launch_fwd_general<true>(C, dim3(total_tiles), stream, 0, (const float2 *)uv, conic, opacity, feature,
                             idx_sorted, (const int2 *)tile_range, bg, 1, 1, out, final_T, ncontrib, bb);
    return check_launch("batch_alpha_blending_forward");
}

static int batch_blend_backward(const void *plan, int B, int total_tiles, int64_t rows, int C,
                                int feature_per_camera, const float *uv, const float *conic, const float *opacity,
                                const float *feature, const int32_t *idx_sorted, const int32_t *tile_range, float bg,
                                const float *final_T, const int32_t *ncontrib, const float *dL_dout, float *dL_duv,
                                float *dL_dconic, float *dL_dopacity, float *dL_dfeature,
                                const unsigned char *entry_masks, cudaStream_t stream) {
    if (B <= 0 || total_tiles < 0 || C <= 0 || rows < 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_alpha_blending_backward: bad sizes");
    if (!plan || !uv || !conic || !opacity || !feature || !tile_range || !final_T || !ncontrib || !dL_dout ||
        !dL_duv || !dL_dconic || !dL_dopacity || !dL_dfeature)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_alpha_blending_backward: null pointer");
    if (total_tiles == 0 || rows == 0) return MSPLAT_OK;
    const BlendBatch bb{batch_plan_view(plan, B), feature_per_camera};
    if (C <= 4) {
        dispatch_small_batch(true, C, total_tiles, stream, bb, (const float2 *)uv, conic, opacity, feature, idx_sorted,
                             (const int2 *)tile_range, bg, nullptr, nullptr, nullptr, final_T, ncontrib, dL_dout,
                             dL_duv, dL_dconic, dL_dopacity, dL_dfeature, const_cast<unsigned char *>(entry_masks));
        launch(batch_blend_grad_finish_kernel, (unsigned)ceil_div64(rows, 256), 256, 0, stream, bb.pv, rows, conic,
               opacity, dL_duv, dL_dconic);
        return check_launch("batch_alpha_blending_backward");
    }
    if (C <= kWideMaxC) {
        launch_bwd_wide<true>(C, dim3(total_tiles), stream, 0, (const float2 *)uv, conic, opacity, feature, idx_sorted,
                              (const int2 *)tile_range, bg, 1, 1, final_T, ncontrib, dL_dout, dL_duv, dL_dconic,
                              dL_dopacity, dL_dfeature, bb);
        return check_launch("batch_alpha_blending_backward");
    }
    for (int c0 = 0; c0 < C; c0 += kBwdC)
        launch(blend_bwd_kernel<true>, total_tiles, kBlendThreads, 0, stream, 0, C, c0, (const float2 *)uv, conic,
               opacity, feature, idx_sorted, (const int2 *)tile_range, bg, 1, 1, final_T, ncontrib, dL_dout, dL_duv,
               dL_dconic, dL_dopacity, dL_dfeature, bb);
    return check_launch("batch_alpha_blending_backward");
}

extern "C" int msplat_batch_alpha_blending_forward(const void *plan, int B, int total_tiles, int C,
                                                   int feature_per_camera, const float *uv, const float *conic,
                                                   const float *opacity, const float *feature,
                                                   const int32_t *idx_sorted, const int32_t *tile_range, float bg,
                                                   float *out, float *final_T, int32_t *ncontrib,
                                                   msplat_stream_t stream) {
    return batch_blend_forward(plan, B, total_tiles, C, feature_per_camera, uv, conic, opacity, feature, idx_sorted,
                               tile_range, bg, out, final_T, ncontrib, nullptr, stream);
}

extern "C" int msplat_batch_alpha_blending_forward_masks(const void *plan, int B, int total_tiles, int C,
                                                         int feature_per_camera, const float *uv, const float *conic,
                                                         const float *opacity, const float *feature,
                                                         const int32_t *idx_sorted, const int32_t *tile_range,
                                                         float bg, float *out, float *final_T, int32_t *ncontrib,
                                                         unsigned char *entry_masks, msplat_stream_t stream) {
    return batch_blend_forward(plan, B, total_tiles, C, feature_per_camera, uv, conic, opacity, feature, idx_sorted,
                               tile_range, bg, out, final_T, ncontrib, entry_masks, stream);
}

extern "C" int msplat_batch_alpha_blending_backward(const void *plan, int B, int total_tiles, int64_t rows, int C,
                                                    int feature_per_camera, const float *uv, const float *conic,
                                                    const float *opacity, const float *feature,
                                                    const int32_t *idx_sorted, const int32_t *tile_range, float bg,
                                                    const float *final_T, const int32_t *ncontrib,
                                                    const float *dL_dout, float *dL_duv, float *dL_dconic,
                                                    float *dL_dopacity, float *dL_dfeature,
                                                    msplat_stream_t stream) {
    return batch_blend_backward(plan, B, total_tiles, rows, C, feature_per_camera, uv, conic, opacity, feature,
                                idx_sorted, tile_range, bg, final_T, ncontrib, dL_dout, dL_duv, dL_dconic,
                                dL_dopacity, dL_dfeature, nullptr, stream);
}

extern "C" int msplat_batch_alpha_blending_backward_masks(const void *plan, int B, int total_tiles, int64_t rows,
                                                          int C, int feature_per_camera, const float *uv,
                                                          const float *conic, const float *opacity,
                                                          const float *feature, const int32_t *idx_sorted,
                                                          const int32_t *tile_range, float bg, const float *final_T,
                                                          const int32_t *ncontrib, const float *dL_dout,
                                                          float *dL_duv, float *dL_dconic, float *dL_dopacity,
                                                          float *dL_dfeature, const unsigned char *entry_masks,
                                                          msplat_stream_t stream) {
    return batch_blend_backward(plan, B, total_tiles, rows, C, feature_per_camera, uv, conic, opacity, feature,
                                idx_sorted, tile_range, bg, final_T, ncontrib, dL_dout, dL_duv, dL_dconic,
                                dL_dopacity, dL_dfeature, entry_masks, stream);
}

extern "C" int msplat_set_blend_ring(int producer_warps, int batch_producer_warps) {
    if ((producer_warps != 0 && producer_warps != 2 && producer_warps != 4) ||
        (batch_producer_warps != 0 && batch_producer_warps != 2 && batch_producer_warps != 4))
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "set_blend_ring: producer warps must be 0, 2 or 4");
    g_fwd_ring = producer_warps;
    g_batch_fwd_ring = batch_producer_warps;
    return MSPLAT_OK;
}

extern "C" int msplat_set_blend_ring_bwd(int producer_warps, int batch_producer_warps) {
    if (producer_warps < 0 || producer_warps > 2 || batch_producer_warps < 0 || batch_producer_warps > 2)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "set_blend_ring_bwd: producer warps must be 0, 1 or 2");
    g_bwd_ring = producer_warps;
    g_batch_bwd_ring = batch_producer_warps;
    return MSPLAT_OK;
}

extern "C" int msplat_set_wait_limit(int polls) {
    if (polls < 0) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "set_wait_limit: polls < 0");
    g_wait_limit = polls;
    return MSPLAT_OK;
}

namespace msplat {
int wait_limit_polls() { return g_wait_limit; }
// The look-back error words of the two translation units that sort.
cudaError_t sort_wait_error_single(int reset, int *value, cudaStream_t stream);
cudaError_t sort_wait_error_batch(int reset, int *value, cudaStream_t stream);
// The bulk-staging error word of the SH kernels.
cudaError_t sh_wait_error(int reset, int *value, cudaStream_t stream);
}  // namespace msplat

extern "C" int msplat_wait_error(int reset, int *error, msplat_stream_t stream) {
    int h = 0;
    cudaError_t e = cudaMemcpyFromSymbolAsync(&h, g_wait_error, sizeof(int), 0, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e == cudaSuccess && reset) {
        const int zero = 0;
        e = cudaMemcpyToSymbolAsync(g_wait_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    }
    int s1 = 0, s2 = 0, s3 = 0;
    if (e == cudaSuccess) e = sort_wait_error_single(reset, &s1, stream);
    if (e == cudaSuccess) e = sort_wait_error_batch(reset, &s2, stream);
    if (e == cudaSuccess) e = sh_wait_error(reset, &s3, stream);
    if (e != cudaSuccess) return set_error(MSPLAT_ERR_LAUNCH, "wait_error: %s", cudaGetErrorString(e));
    const int any = h | s1 | s2 | s3;
    if (error) *error = any;
    if (!any) return MSPLAT_OK;
    return set_error(MSPLAT_ERR_TIMEOUT, "a bounded device-side wait gave up (%s)",
                     h ? "blend ring" : (s1 | s2) ? "sort look-back" : "SH bulk staging");
}
