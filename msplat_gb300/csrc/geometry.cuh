// Per-Gaussian geometry of the rasteriser -- projection, 3-D covariance and
// EWA splatting, forward and adjoint -- as device functions shared by the
// single-stage kernels (project_point.cu, compute_cov3d.cu, ewa_project.cu)
// and the fused preprocess kernels (rasterize.cu).  One source for both
// keeps the fused path bit-identical to the stage-by-stage one.
//
// References: msplat/src/project_point.cu:13-145,
// msplat/src/compute_cov3d.cu:14-147, msplat/src/ewa_project.cu:16-252.
#pragma once

#include "camgrad.cuh"
#include "mat3.cuh"

namespace msplat {

struct Cam {
    float e[12];  // row-major [R | T], world -> camera
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

// ------------------------------------------------------------ projection
// uv = (fx tx / tz + cx - 0.5, fy ty / tz + cy - 0.5), depth = tz, with the
// reference's mixed float/double arithmetic (1/(tz + 1e-7) and the -0.5 in
// double) and expression shape (so the same products contract into FMAs).
// Culled points get uv = 0 and depth = 0.
__device__ __forceinline__ void project_fwd_one(const Cam &c, float px, float py, float pz, int W, int H,
                                                float nearest, float extent, float2 &uv, float &depth) {
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
    uv = culled ? make_float2(0.0f, 0.0f) : make_float2(u, v);
    depth = culled ? 0.0f : tz;
}

// Adjoint of the projection for a point with depth != 0: dL/dxyz and, if
// cam, the camera terms added to acc = [fx, fy, cx, cy, extr[0..11]].
__device__ __forceinline__ void project_bwd_one(const Cam &c, float px, float py, float pz, float2 g, float gd,
                                                float (&dxyz)[3], bool cam, float (&acc)[kCamGradVals]) {
    const float tx = c.e[0] * px + c.e[1] * py + c.e[2] * pz + c.e[3];
    const float ty = c.e[4] * px + c.e[5] * py + c.e[6] * pz + c.e[7];
    const float tz = c.e[8] * px + c.e[9] * py + c.e[10] * pz + c.e[11];
    const float iz = (float)(1.0 / (double)tz);
    const float iz2 = (float)(1.0 / (double)(tz * tz));
    // dL/dt for t = R x + T.
    const float dtx = c.fx * iz * g.x;
    const float dty = c.fy * iz * g.y;
    const float dtz = -(c.fx * tx * g.x + c.fy * ty * g.y) * iz2 + gd;
    dxyz[0] = c.e[0] * dtx + c.e[4] * dty + c.e[8] * dtz;
    dxyz[1] = c.e[1] * dtx + c.e[5] * dty + c.e[9] * dtz;
    dxyz[2] = c.e[2] * dtx + c.e[6] * dty + c.e[10] * dtz;
    if (cam) {
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

// ------------------------------------------------------------ covariance
// glm-style column-major rotation of q = (r, x, y, z) (not normalised: the
// quaternion is taken as unit length, like the reference).
__device__ __forceinline__ Mat3 quat_to_rot_cols(float r, float x, float y, float z) {
    return Mat3::cols(1.f - 2.f * (y * y + z * z), 2.f * (x * y - r * z), 2.f * (x * z + r * y),
                      2.f * (x * y + r * z), 1.f - 2.f * (x * x + z * z), 2.f * (y * z - r * x),
                      2.f * (x * z - r * y), 2.f * (y * z + r * x), 1.f - 2.f * (x * x + y * y));
}

__device__ __forceinline__ Mat3 diag_scale(float sx, float sy, float sz) {
    return Mat3::cols(sx, 0.f, 0.f, 0.f, sy, 0.f, 0.f, 0.f, sz);
}

// Sigma = M^T M with M = S R, upper triangle [s00, s01, s02, s11, s12, s22].
__device__ __forceinline__ void cov3d_fwd_one(float sx, float sy, float sz, float4 q, float (&out)[6]) {
    const Mat3 S = diag_scale(sx, sy, sz);
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

// Adjoint of cov3d_fwd_one given dL/dSigma as the 6-vector (off-diagonal
// entries stand for both (i,j) and (j,i)).
__device__ __forceinline__ void cov3d_bwd_one(const float (&s)[3], float4 q, const float *g, float (&ds)[3],
                                              float4 &dq) {
    const float r = q.x, x = q.y, y = q.z, z = q.w;
    // Standard rotation Rs(i,j); the glm matrix of the forward is its
    // transpose, so M(i,j) = s_i * Rs(j,i) and Sigma = Rs S^2 Rs^T.
    float Rs[3][3];
    Rs[0][0] = 1.f - 2.f * (y * y + z * z); Rs[0][1] = 2.f * (x * y - r * z); Rs[0][2] = 2.f * (x * z + r * y);
    Rs[1][0] = 2.f * (x * y + r * z); Rs[1][1] = 1.f - 2.f * (x * x + z * z); Rs[1][2] = 2.f * (y * z - r * x);
    Rs[2][0] = 2.f * (x * z - r * y); Rs[2][1] = 2.f * (y * z + r * x); Rs[2][2] = 1.f - 2.f * (x * x + y * y);
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

// ------------------------------------------------------------------- EWA
// Camera-space centre, J = d(uv)/d(t), W (rotation of the extrinsics),
// T = J W and the dilated 2-D covariance (a, b, c) = (cov2D00 + 0.3,
// cov2D01, cov2D11 + 0.3), cov2D = T V T^T with glm's summation shape.
struct EwaGeom {
    float tx, ty, tz;
    Mat3 J, Wm, T;
    float a, b, c;
};

__device__ __forceinline__ EwaGeom ewa_geometry(const Cam &k, float px, float py, float pz, const float *v) {
    EwaGeom g;
    g.tx = k.e[0] * px + k.e[1] * py + k.e[2] * pz + k.e[3];
    g.ty = k.e[4] * px + k.e[5] * py + k.e[6] * pz + k.e[7];
    g.tz = k.e[8] * px + k.e[9] * py + k.e[10] * pz + k.e[11];
    g.J = Mat3::cols(k.fx / g.tz, 0.0f, 0.0f,
                     0.0f, k.fy / g.tz, 0.0f,
                     -(k.fx * g.tx) / (g.tz * g.tz), -(k.fy * g.ty) / (g.tz * g.tz), 0.0f);
    g.Wm = Mat3::cols(k.e[0], k.e[4], k.e[8], k.e[1], k.e[5], k.e[9], k.e[2], k.e[6], k.e[10]);
    g.T = g.J * g.Wm;
    const Mat3 V = Mat3::cols(v[0], v[1], v[2], v[1], v[3], v[4], v[2], v[4], v[5]);
    const Mat3 cov2 = g.T * V * g.T.transposed();
    g.a = cov2.c[0][0] + 0.3f;
    g.b = cov2.c[0][1];
    g.c = cov2.c[1][1] + 0.3f;
    return g;
}

// EWA forward of one visible point: det == 0 or an empty tile rectangle
// leave conic / radius / tiles at zero.  lambda = mid +- sqrt(max(0.1,
// mid^2 - det)), radius = ceil(3 sqrt(max lambda)), the rectangle from
// tile_rect (the reference's get_rect).
__device__ __forceinline__ void ewa_fwd_one(const Cam &k, float px, float py, float pz, const float *v, float2 p,
                                            int gx, int gy, float (&conic)[3], int &rad, int &nt) {
    const EwaGeom g = ewa_geometry(k, px, py, pz, v);
    const float det = g.a * g.c - g.b * g.b;
    if (det == 0.0f) return;
    const float mid = 0.5f * (g.a + g.c);
    const float l1 = mid + sqrtf(fmaxf(0.1f, mid * mid - det));
    const float l2 = mid - sqrtf(fmaxf(0.1f, mid * mid - det));
    const float r = ceilf(3.f * sqrtf(fmaxf(l1, l2)));
    int x0, y0, x1, y1;
    tile_rect(p.x, p.y, (int)r, gx, gy, x0, y0, x1, y1);
    const int area = (x1 - x0) * (y1 - y0);
    if (area == 0) return;
    const float inv_det = 1.f / det;
    conic[0] = g.c * inv_det;
    conic[1] = -g.b * inv_det;
    conic[2] = g.a * inv_det;
    rad = (int)r;
    nt = area;
}

// EWA adjoint of one point with radius > 0: given dL/dconic, writes
// dL/dxyz and dL/dV (the 6-vector convention of cov3d_bwd_one) and, if cam,
// adds the camera terms to acc.  Returns false (outputs untouched) when
// det == 0, where the forward left the point invisible.
__device__ __forceinline__ bool ewa_bwd_one(const Cam &k, float px, float py, float pz, const float *v,
                                            float gc0, float gc1, float gc2, float (&dxyz)[3], float (&dV)[6],
                                            bool cam, float (&acc)[kCamGradVals]) {
    const EwaGeom g = ewa_geometry(k, px, py, pz, v);
    const float det = g.a * g.c - g.b * g.b;
    if (det == 0.0f) return false;
    // conic = (c, -b, a) / det with det = a c - b^2.
    const float inv2 = 1.0f / (det * det);
    const float da = inv2 * (-g.c * g.c * gc0 + g.b * g.c * gc1 + (det - g.a * g.c) * gc2);
    const float db = inv2 * (2.f * g.b * g.c * gc0 - (det + 2.f * g.b * g.b) * gc1 + 2.f * g.a * g.b * gc2);
    const float dc = inv2 * ((det - g.a * g.c) * gc0 + g.a * g.b * gc1 - g.a * g.a * gc2);
    // Rows 0 and 1 of T in maths order: T0[k] = T(0,k), T1[k] = T(1,k).
    float T0[3], T1[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        T0[q] = g.T.c[q][0];
        T1[q] = g.T.c[q][1];
    }
    const float Vm[3][3] = {{v[0], v[1], v[2]}, {v[1], v[3], v[4]}, {v[2], v[4], v[5]}};
    // cov2D(0,0) = T0 V T0, cov2D(0,1) = T0 V T1, cov2D(1,1) = T1 V T1.
    dV[0] = T0[0] * T0[0] * da + T0[0] * T1[0] * db + T1[0] * T1[0] * dc;
    dV[3] = T0[1] * T0[1] * da + T0[1] * T1[1] * db + T1[1] * T1[1] * dc;
    dV[5] = T0[2] * T0[2] * da + T0[2] * T1[2] * db + T1[2] * T1[2] * dc;
    dV[1] = 2.f * T0[0] * T0[1] * da + (T0[0] * T1[1] + T0[1] * T1[0]) * db + 2.f * T1[0] * T1[1] * dc;
    dV[2] = 2.f * T0[0] * T0[2] * da + (T0[0] * T1[2] + T0[2] * T1[0]) * db + 2.f * T1[0] * T1[2] * dc;
    dV[4] = 2.f * T0[1] * T0[2] * da + (T0[1] * T1[2] + T0[2] * T1[1]) * db + 2.f * T1[1] * T1[2] * dc;
    float VT0[3], VT1[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        VT0[q] = Vm[q][0] * T0[0] + Vm[q][1] * T0[1] + Vm[q][2] * T0[2];
        VT1[q] = Vm[q][0] * T1[0] + Vm[q][1] * T1[1] + Vm[q][2] * T1[2];
    }
    float dT0[3], dT1[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        dT0[q] = 2.f * VT0[q] * da + VT1[q] * db;
        dT1[q] = VT0[q] * db + 2.f * VT1[q] * dc;
    }
    // T = J R: T(0,:) = J00 R0 + J02 R2, T(1,:) = J11 R1 + J12 R2.
    const float *R0 = k.e, *R1 = k.e + 4, *R2 = k.e + 8;
    const float dJ00 = R0[0] * dT0[0] + R0[1] * dT0[1] + R0[2] * dT0[2];
    const float dJ02 = R2[0] * dT0[0] + R2[1] * dT0[1] + R2[2] * dT0[2];
    const float dJ11 = R1[0] * dT1[0] + R1[1] * dT1[1] + R1[2] * dT1[2];
    const float dJ12 = R2[0] * dT1[0] + R2[1] * dT1[1] + R2[2] * dT1[2];
    const float iz = 1.f / g.tz, iz2 = iz * iz, iz3 = iz2 * iz;
    const float dtx = -k.fx * iz2 * dJ02;
    const float dty = -k.fy * iz2 * dJ12;
    const float dtz = -k.fx * iz2 * dJ00 - k.fy * iz2 * dJ11 + 2.f * k.fx * g.tx * iz3 * dJ02 +
                      2.f * k.fy * g.ty * iz3 * dJ12;
    dxyz[0] = R0[0] * dtx + R1[0] * dty + R2[0] * dtz;
    dxyz[1] = R0[1] * dtx + R1[1] * dty + R2[1] * dtz;
    dxyz[2] = R0[2] * dtx + R1[2] * dty + R2[2] * dtz;
    if (cam) {
        const float J00 = g.J.c[0][0], J11 = g.J.c[1][1];
        const float J02 = g.J.c[2][0], J12 = g.J.c[2][1];
        acc[0] += iz * dJ00 - g.tx * iz2 * dJ02;
        acc[1] += iz * dJ11 - g.ty * iz2 * dJ12;
        const float pt[3] = {px, py, pz};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            // Through T = J R ...
            acc[4 + q] += J00 * dT0[q];
            acc[8 + q] += J11 * dT1[q];
            acc[12 + q] += J02 * dT0[q] + J12 * dT1[q];
            // ... and through t = R x + T.
            acc[4 + q] += pt[q] * dtx;
            acc[8 + q] += pt[q] * dty;
            acc[12 + q] += pt[q] * dtz;
        }
        acc[7] += dtx;
        acc[11] += dty;
        acc[15] += dtz;
    }
    return true;
}

}  // namespace msplat
