// Device math for the FEM hot path: float3 / 3x3 helpers, the principal-stretch
// clamp and the scale-normalised 3x3 block inverse.  Everything is plain
// float32 arithmetic written out here; no CUDA math-library internals are used.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace fem {

struct M3 {
    float m[3][3];  // row-major: m[row][col]
};

__host__ __device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ float len3(float3 a) { return sqrtf(dot3(a, a)); }
__host__ __device__ __forceinline__ float3 xyz(float4 a) { return f3(a.x, a.y, a.z); }
__host__ __device__ __forceinline__ float4 f4(float3 a) { return make_float4(a.x, a.y, a.z, 0.0f); }

__host__ __device__ __forceinline__ float det3(const M3& a) {
    return a.m[0][0] * (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1]) -
           a.m[0][1] * (a.m[1][0] * a.m[2][2] - a.m[1][2] * a.m[2][0]) +
           a.m[0][2] * (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]);
}

__host__ __device__ __forceinline__ float3 col(const M3& a, int c) { return f3(a.m[0][c], a.m[1][c], a.m[2][c]); }
__host__ __device__ __forceinline__ float3 row(const M3& a, int r) { return f3(a.m[r][0], a.m[r][1], a.m[r][2]); }

__host__ __device__ __forceinline__ float3 mul(const M3& a, float3 v) {
    return f3(a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z, a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z,
              a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z);
}

// Transposed product a^T v.
__host__ __device__ __forceinline__ float3 mulT(const M3& a, float3 v) {
    return f3(a.m[0][0] * v.x + a.m[1][0] * v.y + a.m[2][0] * v.z, a.m[0][1] * v.x + a.m[1][1] * v.y + a.m[2][1] * v.z,
              a.m[0][2] * v.x + a.m[1][2] * v.y + a.m[2][2] * v.z);
}

__host__ __device__ __forceinline__ M3 matmul(const M3& a, const M3& b) {
    M3 c;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) c.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
    return c;
}

// a * b^T
__host__ __device__ __forceinline__ M3 matmulT(const M3& a, const M3& b) {
    M3 c;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) c.m[i][j] = a.m[i][0] * b.m[j][0] + a.m[i][1] * b.m[j][1] + a.m[i][2] * b.m[j][2];
    return c;
}

__host__ __device__ __forceinline__ M3 from_cols(float3 a, float3 b, float3 c) {
    M3 r;
    r.m[0][0] = a.x; r.m[0][1] = b.x; r.m[0][2] = c.x;
    r.m[1][0] = a.y; r.m[1][1] = b.y; r.m[1][2] = c.y;
    r.m[2][0] = a.z; r.m[2][1] = b.z; r.m[2][2] = c.z;
    return r;
}

// ---------------------------------------------------------------------------
// Signed 3x3 SVD and the principal-stretch clamp.
//
// Method: cyclic Jacobi eigen-decomposition of the symmetric C = F^T F
// (Golub & Van Loan, Matrix Computations, sec. 8.5), V from the rotations,
// U by normalising F v_1, Gram-Schmidt on F v_2 and u_3 = u_1 x u_2, so that
// U and V are proper rotations and the smallest stretch carries sign(det F) --
// the rotation-variant convention of Irving et al. 2004 and McAdams et al.
// 2011 that the reference's clamp is written against (an inverted element has
// a negative smallest stretch and the clamp lifts it to min_stretch).
// ---------------------------------------------------------------------------

__device__ __forceinline__ void jacobi_rotate(float (&c)[3][3], float (&v)[3][3], int p, int q) {
    float apq = c[p][q];
    if (fabsf(apq) < 1e-30f) return;
    float app = c[p][p], aqq = c[q][q];
    float tau = (aqq - app) / (2.0f * apq);
    float t = copysignf(1.0f, tau) / (fabsf(tau) + sqrtf(1.0f + tau * tau));
    float cs = rsqrtf(1.0f + t * t);
    float sn = t * cs;
    // C' = J^T C J with J the (p,q) Givens rotation
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float ckp = c[k][p], ckq = c[k][q];
        c[k][p] = cs * ckp - sn * ckq;
        c[k][q] = sn * ckp + cs * ckq;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float cpk = c[p][k], cqk = c[q][k];
        c[p][k] = cs * cpk - sn * cqk;
        c[q][k] = sn * cpk + cs * cqk;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float vkp = v[k][p], vkq = v[k][q];
        v[k][p] = cs * vkp - sn * vkq;
        v[k][q] = sn * vkp + cs * vkq;
    }
}

// F = U diag(s) V^T with U, V rotations, s0 >= s1 >= |s2|, s2 signed.
__device__ inline void signed_svd(const M3& F, M3& U, float3& s, M3& V) {
    float c[3][3], v[3][3] = {{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            c[i][j] = F.m[0][i] * F.m[0][j] + F.m[1][i] * F.m[1][j] + F.m[2][i] * F.m[2][j];
    for (int sweep = 0; sweep < 6; ++sweep) {
        jacobi_rotate(c, v, 0, 1);
        jacobi_rotate(c, v, 0, 2);
        jacobi_rotate(c, v, 1, 2);
    }
    float ev[3] = {c[0][0], c[1][1], c[2][2]};
    int o0 = 0, o1 = 1, o2 = 2;  // sort descending
    if (ev[o0] < ev[o1]) { int t = o0; o0 = o1; o1 = t; }
    if (ev[o1] < ev[o2]) { int t = o1; o1 = o2; o2 = t; }
    if (ev[o0] < ev[o1]) { int t = o0; o0 = o1; o1 = t; }
    float3 v0 = f3(v[0][o0], v[1][o0], v[2][o0]);
    float3 v1 = f3(v[0][o1], v[1][o1], v[2][o1]);
    float3 v2 = cross3(v0, v1);  // proper rotation V
    float3 b0 = mul(F, v0), b1 = mul(F, v1), b2 = mul(F, v2);
    float s0 = len3(b0);
    float3 u0 = s0 > 1e-30f ? b0 * (1.0f / s0) : f3(1.f, 0.f, 0.f);
    float3 w1 = b1 - u0 * dot3(u0, b1);
    float s1 = len3(w1);
    float3 u1;
    if (s1 > 1e-30f) {
        u1 = w1 * (1.0f / s1);
    } else {  // any unit vector orthogonal to u0
        float3 t = fabsf(u0.x) < 0.9f ? f3(1.f, 0.f, 0.f) : f3(0.f, 1.f, 0.f);
        u1 = cross3(u0, t);
        u1 = u1 * (1.0f / len3(u1));
    }
    float3 u2 = cross3(u0, u1);
    float s2 = dot3(u2, b2);
    U = from_cols(u0, u1, u2);
    V = from_cols(v0, v1, v2);
    s = f3(s0, s1, s2);
}

// Principal-stretch clamp (reference kernels.py:421-444).  Returns F unchanged
// when a bound is negative or when all signed stretches already lie inside
// [lo, hi]; the in-range test uses sigma_max^2 <= ||F||_F^2 and
// sigma_min >= 2 det(F) / ||F||_F^2 (from lambda_min >= det(C)/(lambda_1 lambda_2)),
// a sufficient condition that avoids the decomposition for ordinary elements.
__device__ inline M3 clamp_stretch(const M3& F, float lo, float hi) {
    if (lo < 0.0f || hi < 0.0f) return F;
    float ic = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) ic += F.m[i][j] * F.m[i][j];
    float J = det3(F);
    if (J > 0.0f && ic <= hi * hi && 2.0f * J >= lo * ic) return F;
    M3 U, V;
    float3 s;
    signed_svd(F, U, s, V);
    s.x = fmaxf(fminf(s.x, hi), lo);
    s.y = fmaxf(fminf(s.y, hi), lo);
    s.z = fmaxf(fminf(s.z, hi), lo);
    M3 out;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            out.m[i][j] = U.m[i][0] * s.x * V.m[j][0] + U.m[i][1] * s.y * V.m[j][1] + U.m[i][2] * s.z * V.m[j][2];
    return out;
}

// Scale-normalised inverse of a diagonal block with point-Jacobi fallback
// (reference kernels.py:1817-1833).  The inverse of the normalised block is
// its adjugate over its determinant.
__device__ __forceinline__ void inverse_diagonal_block(const float* blk, float* out) {
    float scale = fmaxf(fabsf(blk[0]), fmaxf(fabsf(blk[4]), fabsf(blk[8])));
    if (scale > 0.0f) {
        float a[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) a[k] = blk[k] / scale;
        float trace = (a[0] + a[4] + a[8]) / 3.0f;
        float c00 = a[4] * a[8] - a[5] * a[7];
        float c01 = a[5] * a[6] - a[3] * a[8];
        float c02 = a[3] * a[7] - a[4] * a[6];
        float det = a[0] * c00 + a[1] * c01 + a[2] * c02;
        if (trace > 0.0f && fabsf(det) > 1.0e-9f * trace * trace * trace) {
            float id = 1.0f / det;
            out[0] = c00 * id / scale;
            out[1] = (a[2] * a[7] - a[1] * a[8]) * id / scale;
            out[2] = (a[1] * a[5] - a[2] * a[4]) * id / scale;
            out[3] = c01 * id / scale;
            out[4] = (a[0] * a[8] - a[2] * a[6]) * id / scale;
            out[5] = (a[2] * a[3] - a[0] * a[5]) * id / scale;
            out[6] = c02 * id / scale;
            out[7] = (a[1] * a[6] - a[0] * a[7]) * id / scale;
            out[8] = (a[0] * a[4] - a[1] * a[3]) * id / scale;
            return;
        }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) out[k] = 0.0f;
    out[0] = blk[0] > 0.0f ? 1.0f / blk[0] : 1.0f;
    out[4] = blk[4] > 0.0f ? 1.0f / blk[4] : 1.0f;
    out[8] = blk[8] > 0.0f ? 1.0f / blk[8] : 1.0f;
}

// Point-Jacobi inverse of the scalar diagonal: 1/d, or 1 where d == 0.
__device__ __forceinline__ void inverse_point_diagonal(const float* blk, float* out) {
#pragma unroll
    for (int k = 0; k < 9; ++k) out[k] = 0.0f;
    out[0] = blk[0] != 0.0f ? 1.0f / blk[0] : 1.0f;
    out[4] = blk[4] != 0.0f ? 1.0f / blk[4] : 1.0f;
    out[8] = blk[8] != 0.0f ? 1.0f / blk[8] : 1.0f;
}

}  // namespace fem
