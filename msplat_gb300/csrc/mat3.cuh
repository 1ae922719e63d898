// A column-major 3x3 float matrix with the arithmetic of the header-only
// glm library, which the reference uses for its covariance and EWA maths
// (msplat/src/compute_cov3d.cu:14-117, msplat/src/ewa_project.cu:41-59).
//
// m.c[j][i] is column j, row i.  The product evaluates every entry as the
// left-to-right sum a0*b0 + a1*b1 + a2*b2 over the shared index (zeros
// included), which is how glm's mat3 operator* is written; keeping that
// exact expression shape lets the compiler make the same FMA contractions,
// so covariances, radii and tile counts come out bit-identical.
#pragma once

namespace msplat {

struct Mat3 {
    float c[3][3];

    // Column-major constructor from nine values (column 0 first), like glm.
    __device__ __forceinline__ static Mat3 cols(float a00, float a01, float a02,
                                                float a10, float a11, float a12,
                                                float a20, float a21, float a22) {
        Mat3 m;
        m.c[0][0] = a00; m.c[0][1] = a01; m.c[0][2] = a02;
        m.c[1][0] = a10; m.c[1][1] = a11; m.c[1][2] = a12;
        m.c[2][0] = a20; m.c[2][1] = a21; m.c[2][2] = a22;
        return m;
    }

    __device__ __forceinline__ Mat3 transposed() const {
        Mat3 t;
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int i = 0; i < 3; ++i) t.c[j][i] = c[i][j];
        return t;
    }
};

// (A * B) column j, row i = sum_k A(col k, row i) * B(col j, row k).
__device__ __forceinline__ Mat3 operator*(const Mat3 &A, const Mat3 &B) {
    Mat3 R;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i)
            R.c[j][i] = A.c[0][i] * B.c[j][0] + A.c[1][i] * B.c[j][1] + A.c[2][i] * B.c[j][2];
    return R;
}

}  // namespace msplat
