// Conservative reach tests of a 2-D Gaussian (conic a, b, c around
// (gx, gy), opacity op) against pixel boxes, shared by the blend kernels
// (per tile and per warp block) and by the tile lists of the fused path
// (per Gaussian rectangle).  A box the test rules out holds no pixel centre
// whose alpha = min(0.99, op exp(-q/2)) the blend would find >= 1/255, so
// dropping it changes no blended result.
#pragma once

#include "common.cuh"

namespace msplat {

// The threshold of cull_box: a pixel of the box [gx + lx, gx + hx] x
// [gy + ly, gy + hy] (bx1, by1: its far corner) can reach alpha >= 1/255
// under the blend's float evaluation only where the exact q <= tau + err,
// err bounding how far that evaluation can sit below the exact value:
// product/sum rounding (relative to the term sizes), rounding of the
// coordinate differences (relative to the coordinates), and the
// approximate logarithm in tau.
__device__ __forceinline__ float box_threshold(float gx, float gy, float a, float b, float c, float tau, float lx,
                                               float hx, float ly, float hy, float bx1, float by1) {
    const float DX = fmaxf(fabsf(lx), fabsf(hx)), DY = fmaxf(fabsf(ly), fabsf(hy));
    const float coord_eps = 1e-6f * (fabsf(gx) + fabsf(gy) + fabsf(bx1) + fabsf(by1) + 1.0f);
    const float err = 1e-5f * (a * DX * DX + c * DY * DY + 2.0f * fabsf(b) * DX * DY) +
                      4.0f * coord_eps * (a * DX + c * DY + 2.0f * fabsf(b) * (DX + DY)) +
                      1e-5f * fabsf(tau) + 1e-4f;
    return tau + err;
}

// Conservative test: true only if no pixel centre of the box
// [bx0, bx1] x [by0, by1] can reach alpha >= 1/255 under the blend's float
// evaluation.  L receives the threshold it used: a pixel of the box can
// contribute only where the exact q = a dx^2 + 2 b dx dy + c dy^2 is <= L
// (INFINITY or NaN when the test gives no such bound).
// cull_box for opacity > 0 with tau = 2 log(255 op) given (a caller that
// tests several boxes of one Gaussian computes it once).
__device__ __forceinline__ bool cull_box_tau(float gx, float gy, float a, float b, float c, float tau, float bx0,
                                             float by0, float bx1, float by1, float &L) {
    L = INFINITY;
    const float det = a * c - b * b;
    if (!(a > 0.0f) || !(c > 0.0f) || !(det > 0.0f)) return false;  // not an ellipse
    const float lx = bx0 - gx, hx = bx1 - gx, ly = by0 - gy, hy = by1 - gy;  // pixel - centre
    L = box_threshold(gx, gy, a, b, c, tau, lx, hx, ly, hy, bx1, by1);
    if (lx <= 0.0f && hx >= 0.0f && ly <= 0.0f && hy >= 0.0f) return L < 0.0f;
    // Minimum of q(dx, dy) = a dx^2 + 2 b dx dy + c dy^2 over the box edges.
    float qmin = INFINITY;
    {
        const float xs[2] = {lx, hx};
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const float dx = xs[e];
            const float dy = fminf(fmaxf(-b * dx / c, ly), hy);
            qmin = fminf(qmin, a * dx * dx + 2.0f * b * dx * dy + c * dy * dy);
        }
        const float ys[2] = {ly, hy};
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const float dy = ys[e];
            const float dx = fminf(fmaxf(-b * dy / a, lx), hx);
            qmin = fminf(qmin, a * dx * dx + 2.0f * b * dx * dy + c * dy * dy);
        }
    }
    return qmin > L;
}

__device__ __forceinline__ bool cull_box(float gx, float gy, float a, float b, float c, float op, float bx0,
                                         float by0, float bx1, float by1, float &L) {
    if (!(op > 0.0f)) {  // NaN opacity is never culled
        L = op;
        return op <= 0.0f;
    }
    const float tau = 2.0f * logf(255.0f * op);  // q <= tau  <=>  op e^{-q/2} >= 1/255
    return cull_box_tau(gx, gy, a, b, c, tau, bx0, by0, bx1, by1, L);
}

// The same test for the 16 x 16 tile whose first pixel centre is (bx0, by0).
__device__ __forceinline__ bool cull_tile(float gx, float gy, float a, float b, float c, float op,
                                          float bx0, float by0, float &L) {
    return cull_box(gx, gy, a, b, c, op, bx0, by0, bx0 + (float)(kTile - 1), by0 + (float)(kTile - 1), L);
}

__device__ __forceinline__ bool cull_tile(float gx, float gy, float a, float b, float c, float op,
                                          float bx0, float by0) {
    float L;
    return cull_tile(gx, gy, a, b, c, op, bx0, by0, L);
}

// Images of at least this many tiles (about 1280 x 720 and up) cut each
// rectangle row by row (row_span); smaller ones keep whole rectangles:
// their Gaussians span a row or two, so the cut removes little and its
// arithmetic and two-level emit cost more than the shorter lists save
// (measured on 256 x 256 and 512 x 512 cameras of the multi-camera batch).
constexpr int kRowCutMinTiles = 3000;
__host__ __device__ __forceinline__ bool row_cut_enabled(int gx, int gy) { return gx * gy >= kRowCutMinTiles; }

// What the per-row reach of a Gaussian needs (row_span), computed once per
// Gaussian over its (shrunk) tile rectangle.  From the threshold L of
// cull_box (box_threshold) for the whole rectangle (a pixel of the rectangle can
// contribute only where the exact q <= L; L of a sub-box, such as one
// tile row, is never larger, so the rectangle's L is safe for every row):
// the extents ex = sqrt(L c / det), ey = sqrt(L a / det) of q <= L, the dy
// yr = -b ex / c of its rightmost point, a L, 1 / a, and the x margin.
// The record is written once (by the count kernel) and read by both
// kernels that evaluate row_span, so only row_span itself must be
// evaluated identically in both.
struct RowReach {
    float gx, gy, b, det, ia, aL, ex, ey, yr, mx;
    int usable;  // 0: keep whole rows (nearly degenerate conic, or no usable L)
};

__device__ __forceinline__ RowReach row_reach(float gx, float gy, float a, float b, float c, float op, int x0, int y0,
                                              int x1, int y1) {
    constexpr float T = (float)kTile;
    RowReach r{};
    r.gx = gx;
    r.gy = gy;
    r.b = b;
    r.usable = 0;
    if (!(x0 < x1 && y0 < y1) || !(op > 0.0f)) return r;
    const float tau = 2.0f * logf(255.0f * op);
    const float bx1 = x1 * T - 1.0f, by1 = y1 * T - 1.0f;
    const float L = box_threshold(gx, gy, a, b, c, tau, x0 * T - gx, bx1 - gx, y0 * T - gy, by1 - gy, bx1, by1);
    const float det = a * c - b * b;
    if (!(L >= 0.0f) || !(L < INFINITY) || !(a > 0.0f) || !(c > 0.0f) || !(det >= 0.01f * a * c)) return r;
    r.det = det;
    r.ia = 1.0f / a;
    r.aL = a * L;
    r.ex = sqrtf(L * c / det);
    r.ey = sqrtf(L * a / det);
    r.yr = -b * r.ex / c;
    // widened by 1 % plus 0.05 px and the coordinates' rounding, as in
    // warp_block_mask (the rectangle's farthest column bounds |x|)
    r.mx = 0.01f * r.ex + 0.05f + 4e-6f * (fabsf(gx) + (float)(x1 * kTile) + T);
    r.usable = r.ex == r.ex && r.ey == r.ey && r.yr == r.yr && r.mx == r.mx && r.ia == r.ia;  // no NaN
    return r;
}

// Hardware square root (one instruction, the same result wherever it runs;
// its error of a few ulp is far inside the 1 % margin).
__device__ __forceinline__ float sqrt_hw(float x) {
    float y;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// The columns [xa, xb) of [x0, x1) whose tiles in tile row ty (pixel rows
// 16 ty .. 16 ty + 15) the ellipse q <= L can reach -- the transpose of
// warp_block_mask: per row band the reachable pixel columns are the
// x-extent of the ellipse inside the band; the right boundary
// x(y) = (-b y + sqrt(a L - det y^2)) / a is concave with its maximum ex
// at y = yr, so over the band it peaks there or at the nearer band edge
// (the left boundary mirrors it); a band beyond the ellipse's y-extent ey
// reaches nothing.  Extents are widened as in warp_block_mask.  Every
// operation is exact, an explicitly rounded intrinsic (never contracted)
// or sqrt_hw, so the count kernel and the emit, which both evaluate it on
// the same record, get the same span.
__device__ __forceinline__ void row_span(const RowReach &r, int ty, int x0, int x1, int &xa, int &xb) {
    xa = x0;
    xb = x1;
    if (!r.usable) return;
    const float by0 = (float)(ty * kTile);
    const float ly = __fsub_rn(by0, r.gy), hy = __fadd_rn(ly, (float)(kTile - 1));  // pixel - centre
    const float my = __fadd_rn(__fadd_rn(__fmul_rn(0.01f, r.ey), 0.05f),
                               __fmul_rn(4e-6f, __fadd_rn(__fadd_rn(fabsf(r.gy), fabsf(by0)), (float)kTile)));
    if (hy < __fsub_rn(-r.ey, my) || ly > __fadd_rn(r.ey, my)) {  // the band misses the ellipse
        xb = xa;
        return;
    }
    float right = r.ex, left = -r.ex;
    if (!(r.yr >= ly && r.yr <= hy)) {
        const float y = fminf(fmaxf(r.yr, ly), hy);
        const float d = fmaxf(__fsub_rn(r.aL, __fmul_rn(r.det, __fmul_rn(y, y))), 0.0f);
        right = __fmul_rn(__fadd_rn(__fmul_rn(-r.b, y), sqrt_hw(d)), r.ia);
    }
    if (!(-r.yr >= ly && -r.yr <= hy)) {
        const float y = fminf(fmaxf(-r.yr, ly), hy);
        const float d = fmaxf(__fsub_rn(r.aL, __fmul_rn(r.det, __fmul_rn(y, y))), 0.0f);
        left = __fmul_rn(__fsub_rn(__fmul_rn(-r.b, y), sqrt_hw(d)), r.ia);
    }
    const float lo = __fsub_rn(__fadd_rn(r.gx, left), r.mx), hi = __fadd_rn(__fadd_rn(r.gx, right), r.mx);
    if (!(lo <= hi)) return;  // (NaN: keep the row)
    const float inv_t = 1.0f / (float)kTile;  // a power of two: the products are exact
    const float tlo = floorf(lo * inv_t), thi = floorf(hi * inv_t);
    xa = (int)fminf(fmaxf(tlo, (float)x0), (float)x1);
    xb = (int)fminf(fmaxf(thi + 1.0f, (float)x0), (float)x1);
    if (xb < xa) xb = xa;
}

// The tiles of rectangle [x0, x1) x [y0, y1) the per-row reach keeps.
__device__ __forceinline__ int row_span_count(const RowReach &r, int x0, int y0, int x1, int y1) {
    if (!r.usable) return (x1 - x0) * max(0, y1 - y0);
    int n = 0;
    for (int ty = y0; ty < y1; ++ty) {
        int xa, xb;
        row_span(r, ty, x0, x1, xa, xb);
        n += xb - xa;
    }
    return n;
}

// Shrinks a Gaussian's tile rectangle [x0, x1) x [y0, y1) (tile units) to
// the rows and columns its alpha >= 1/255 ellipse reaches; an empty result
// has x0 == x1 and y0 == y1.  The cut is proposed from the ellipse's
// bounding box (half-extents sqrt(tau a / det) and sqrt(tau c / det),
// widened by 0.2 % + 0.05 px) and a side is cut only if cull_box rules out
// the whole strip cut off, so every dropped tile is one no pixel of which
// the Gaussian reaches; if it does not, the strip one tile narrower is
// tried, and failing that the side stays (the rectangle stays
// conservative, only less tight).  At most eight box tests per Gaussian,
// usually four; none where the box proposes no cut.
__device__ __forceinline__ void shrink_rect(float gx, float gy, float a, float b, float c, float op, int &x0,
                                            int &y0, int &x1, int &y1) {
    constexpr float T = (float)kTile;
    if (x0 >= x1 || y0 >= y1) return;
    float L;
    if (!(op > 0.0f)) {  // op <= 0 reaches nothing; NaN keeps everything
        if (op <= 0.0f) {
            x1 = x0;
            y1 = y0;
        }
        return;
    }
    const float tau = 2.0f * logf(255.0f * op);
    const float det = a * c - b * b;
    if (!(a > 0.0f) || !(c > 0.0f) || !(det > 0.0f)) return;
    if (!(tau > 0.0f)) {  // the ellipse is (nearly) empty: try the whole rectangle
        if (cull_box_tau(gx, gy, a, b, c, tau, x0 * T, y0 * T, x1 * T - 1.0f, y1 * T - 1.0f, L)) {
            x1 = x0;
            y1 = y0;
        }
        return;
    }
    const float ey = 1.002f * sqrtf(tau * a / det) + 0.05f, ex = 1.002f * sqrtf(tau * c / det) + 0.05f;
    // proposed tile range: tiles whose pixel rows / columns meet [g - e, g + e]
    const float fy0 = floorf((gy - ey) / T), fy1 = floorf((gy + ey) / T) + 1.0f;
    const float fx0 = floorf((gx - ex) / T), fx1 = floorf((gx + ex) / T) + 1.0f;
    if (!(fy0 == fy0) || !(fx0 == fx0) || !(fy1 == fy1) || !(fx1 == fx1)) return;  // NaN
    const int py0 = (int)fmaxf(fy0, (float)y0), py1 = (int)fminf(fy1, (float)y1);
    const int px0 = (int)fmaxf(fx0, (float)x0), px1 = (int)fminf(fx1, (float)x1);
    if (py0 >= py1 || px0 >= px1) {  // the box misses the rectangle: try all of it
        if (cull_box_tau(gx, gy, a, b, c, tau, x0 * T, y0 * T, x1 * T - 1.0f, y1 * T - 1.0f, L)) {
            x1 = x0;
            y1 = y0;
        }
        return;
    }
    for (int k = py0; k > y0 && k >= py0 - 1; --k)
        if (cull_box_tau(gx, gy, a, b, c, tau, x0 * T, y0 * T, x1 * T - 1.0f, k * T - 1.0f, L)) {
            y0 = k;
            break;
        }
    for (int k = py1; k < y1 && k <= py1 + 1; ++k)
        if (cull_box_tau(gx, gy, a, b, c, tau, x0 * T, k * T, x1 * T - 1.0f, y1 * T - 1.0f, L)) {
            y1 = k;
            break;
        }
    for (int k = px0; k > x0 && k >= px0 - 1; --k)
        if (cull_box_tau(gx, gy, a, b, c, tau, x0 * T, y0 * T, k * T - 1.0f, y1 * T - 1.0f, L)) {
            x0 = k;
            break;
        }
    for (int k = px1; k < x1 && k <= px1 + 1; ++k)
        if (cull_box_tau(gx, gy, a, b, c, tau, k * T, y0 * T, x1 * T - 1.0f, y1 * T - 1.0f, L)) {
            x1 = k;
            break;
        }
}

}  // namespace msplat
