// Conservative reach tests of a 2-D Gaussian (conic a, b, c around
// (gx, gy), opacity op) against pixel boxes, shared by the blend kernels
// (per tile and per warp block) and by the tile lists of the fused path
// (per Gaussian rectangle).  A box the test rules out holds no pixel centre
// whose alpha = min(0.99, op exp(-q/2)) the blend would find >= 1/255, so
// dropping it changes no blended result.
#pragma once

#include "common.cuh"

namespace msplat {

// Conservative test: true only if no pixel centre of the box
// [bx0, bx1] x [by0, by1] can reach alpha >= 1/255 under the blend's float
// evaluation.  L receives the threshold it used: a pixel of the box can
// contribute only where the exact q = a dx^2 + 2 b dx dy + c dy^2 is <= L
// (INFINITY or NaN when the test gives no such bound).
__device__ __forceinline__ bool cull_box(float gx, float gy, float a, float b, float c, float op, float bx0,
                                         float by0, float bx1, float by1, float &L) {
    L = INFINITY;
    if (!(op > 0.0f)) {  // NaN opacity is never culled
        L = op;
        return op <= 0.0f;
    }
    const float tau = 2.0f * logf(255.0f * op);    // q <= tau  <=>  op e^{-q/2} >= 1/255
    const float det = a * c - b * b;
    if (!(a > 0.0f) || !(c > 0.0f) || !(det > 0.0f)) return false;  // not an ellipse
    const float lx = bx0 - gx, hx = bx1 - gx, ly = by0 - gy, hy = by1 - gy;  // pixel - centre
    const float DX = fmaxf(fabsf(lx), fabsf(hx)), DY = fmaxf(fabsf(ly), fabsf(hy));
    // Bound on how far the blend's float evaluation of q at a pixel can sit
    // below the exact value: product/sum rounding (relative to the term
    // sizes), rounding of the coordinate differences (relative to the
    // coordinates), and the approximate logarithm in tau.
    const float coord_eps = 1e-6f * (fabsf(gx) + fabsf(gy) + fabsf(bx1) + fabsf(by1) + 1.0f);
    const float err = 1e-5f * (a * DX * DX + c * DY * DY + 2.0f * fabsf(b) * DX * DY) +
                      4.0f * coord_eps * (a * DX + c * DY + 2.0f * fabsf(b) * (DX + DY)) +
                      1e-5f * fabsf(tau) + 1e-4f;
    L = tau + err;
    if (lx <= 0.0f && hx >= 0.0f && ly <= 0.0f && hy >= 0.0f) return tau + err < 0.0f;
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
    return qmin > tau + err;
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
        if (cull_box(gx, gy, a, b, c, op, x0 * T, y0 * T, x1 * T - 1.0f, y1 * T - 1.0f, L)) {
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
        if (cull_box(gx, gy, a, b, c, op, x0 * T, y0 * T, x1 * T - 1.0f, y1 * T - 1.0f, L)) {
            x1 = x0;
            y1 = y0;
        }
        return;
    }
    for (int k = py0; k > y0 && k >= py0 - 1; --k)
        if (cull_box(gx, gy, a, b, c, op, x0 * T, y0 * T, x1 * T - 1.0f, k * T - 1.0f, L)) {
            y0 = k;
            break;
        }
    for (int k = py1; k < y1 && k <= py1 + 1; ++k)
        if (cull_box(gx, gy, a, b, c, op, x0 * T, k * T, x1 * T - 1.0f, y1 * T - 1.0f, L)) {
            y1 = k;
            break;
        }
    for (int k = px0; k > x0 && k >= px0 - 1; --k)
        if (cull_box(gx, gy, a, b, c, op, x0 * T, y0 * T, k * T - 1.0f, y1 * T - 1.0f, L)) {
            x0 = k;
            break;
        }
    for (int k = px1; k < x1 && k <= px1 + 1; ++k)
        if (cull_box(gx, gy, a, b, c, op, k * T, y0 * T, x1 * T - 1.0f, y1 * T - 1.0f, L)) {
            x1 = k;
            break;
        }
}

}  // namespace msplat
