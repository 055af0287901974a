// Scalar-generic force terms: the triangle membrane (reference kernels.py:876-960)
// and the spring bend torque (kernels.py:221-291) written once over a scalar
// type S.  With S = float they are the forward force; with S = Dual (a value
// and one directional derivative, forward-mode differentiation) one pass per
// input direction gives the exact Jacobian column the adjoint needs, so the
// VJP cannot drift from the force it differentiates.
#pragma once

#include <cuda_runtime.h>

namespace fem {

struct Dual {
    float v, d;
};
__device__ __forceinline__ Dual dual(float v, float d = 0.0f) { return Dual{v, d}; }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual{a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual{a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual{-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual{a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const float q = a.v / b.v;
    return Dual{q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Dual operator+(Dual a, float b) { return Dual{a.v + b, a.d}; }
__device__ __forceinline__ Dual operator-(Dual a, float b) { return Dual{a.v - b, a.d}; }
__device__ __forceinline__ Dual operator-(float a, Dual b) { return Dual{a - b.v, -b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, float b) { return Dual{a.v * b, a.d * b}; }
__device__ __forceinline__ Dual operator*(float a, Dual b) { return Dual{a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, float b) { return Dual{a.v / b, a.d / b}; }

__device__ __forceinline__ float val(float a) { return a; }
__device__ __forceinline__ float val(Dual a) { return a.v; }
__device__ __forceinline__ float gsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ Dual gsqrt(Dual a) {
    const float r = sqrtf(a.v);
    return Dual{r, r > 0.0f ? a.d / (2.0f * r) : 0.0f};
}
__device__ __forceinline__ float gabs(float a) { return fabsf(a); }
__device__ __forceinline__ Dual gabs(Dual a) { return a.v < 0.0f ? -a : a; }
// acos with its argument clamped to [-1, 1] (Warp's acos); zero derivative where clamped
__device__ __forceinline__ float gacos(float a) { return acosf(fminf(fmaxf(a, -1.0f), 1.0f)); }
__device__ __forceinline__ Dual gacos(Dual a) {
    const float c = fminf(fmaxf(a.v, -1.0f), 1.0f);
    const float s = sqrtf(1.0f - c * c);
    return Dual{acosf(c), (a.v > -1.0f && a.v < 1.0f && s > 0.0f) ? -a.d / s : 0.0f};
}
__device__ __forceinline__ float gclamp(float a, float lo, float hi) { return fminf(fmaxf(a, lo), hi); }
__device__ __forceinline__ Dual gclamp(Dual a, float lo, float hi) {
    if (a.v < lo) return Dual{lo, 0.0f};
    if (a.v > hi) return Dual{hi, 0.0f};
    return a;
}

template <class S>
struct V3 {
    S x, y, z;
};
template <class S>
__device__ __forceinline__ V3<S> v3(S x, S y, S z) {
    return V3<S>{x, y, z};
}
template <class S>
__device__ __forceinline__ V3<S> operator+(V3<S> a, V3<S> b) {
    return V3<S>{a.x + b.x, a.y + b.y, a.z + b.z};
}
template <class S>
__device__ __forceinline__ V3<S> operator-(V3<S> a, V3<S> b) {
    return V3<S>{a.x - b.x, a.y - b.y, a.z - b.z};
}
template <class S>
__device__ __forceinline__ V3<S> operator-(V3<S> a) {
    return V3<S>{-a.x, -a.y, -a.z};
}
template <class S, class K>
__device__ __forceinline__ V3<S> operator*(V3<S> a, K k) {
    return V3<S>{a.x * k, a.y * k, a.z * k};
}
template <class S, class K>
__device__ __forceinline__ V3<S> operator/(V3<S> a, K k) {
    return V3<S>{a.x / k, a.y / k, a.z / k};
}
template <class S>
__device__ __forceinline__ S gdot(V3<S> a, V3<S> b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class S>
__device__ __forceinline__ V3<S> gcross(V3<S> a, V3<S> b) {
    return V3<S>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class S>
__device__ __forceinline__ S glength(V3<S> a) {
    return gsqrt(gdot(a, a));
}
// Warp's normalize: a / |a|, the zero vector for |a| = 0
template <class S>
__device__ __forceinline__ V3<S> gnormalize(V3<S> a) {
    const S l = glength(a);
    if (val(l) > 0.0f) return a / l;
    const S z = a.x * 0.0f;
    return V3<S>{z, z, z};
}
template <class S>
__device__ __forceinline__ V3<S> lift3(float3 a) {
    return V3<S>{S(a.x), S(a.y), S(a.z)};
}
template <>
__device__ __forceinline__ V3<Dual> lift3<Dual>(float3 a) {
    return V3<Dual>{dual(a.x), dual(a.y), dual(a.z)};
}

// Triangle membrane force on the three corners (the value each corner's node
// receives): deviatoric P = mu F (I_C - 2)/I_C + k_d dF/dt with F = [x10 x20] Dm,
// the area constraint c = area/area_rest - 1 with its damping, and the
// drag/lift of the mean velocity.  Lame parameters are scaled by the rest
// area 1 / (2 det Dm).  Reference kernels.py:876-960.
template <class S>
__device__ __forceinline__ void triangle_force(const V3<S> x[3], const V3<S> v[3], float4 Dm, const float* mat,
                                               V3<S> out[3]) {
    const float inv_rest_area = (Dm.x * Dm.w - Dm.y * Dm.z) * 2.0f;
    const float rest_area = 1.0f / inv_rest_area;
    const float k_mu = mat[0] * rest_area, k_lambda = mat[1] * rest_area, k_damp = mat[2] * rest_area;
    const float k_drag = mat[3], k_lift = mat[4];
    const V3<S> x10 = x[1] - x[0], x20 = x[2] - x[0];
    const V3<S> v10 = v[1] - v[0], v20 = v[2] - v[0];
    const V3<S> F1 = x10 * Dm.x + x20 * Dm.z, F2 = x10 * Dm.y + x20 * Dm.w;
    const V3<S> dF1 = v10 * Dm.x + v20 * Dm.z, dF2 = v10 * Dm.y + v20 * Dm.w;
    const S Ic = gdot(F1, F1) + gdot(F2, F2);
    const S dev = (Ic - 2.0f) / Ic;
    const V3<S> P1 = F1 * k_mu * dev + dF1 * k_damp;
    const V3<S> P2 = F2 * k_mu * dev + dF2 * k_damp;
    V3<S> f1 = P1 * Dm.x + P2 * Dm.y;
    V3<S> f2 = P1 * Dm.z + P2 * Dm.w;
    V3<S> n = gcross(x10, x20);
    const S area = glength(n) * 0.5f;
    const S c = area * inv_rest_area - 1.0f;
    n = gnormalize(n);
    const V3<S> dcdq = gcross(x20, n) * inv_rest_area * 0.5f;
    const V3<S> dcdr = gcross(n, x10) * inv_rest_area * 0.5f;
    const S f_area = c * k_lambda;
    const S dcdt = gdot(dcdq, v[1]) + gdot(dcdr, v[2]) - gdot(dcdq + dcdr, v[0]);
    const S f_damp = dcdt * k_damp;
    f1 = f1 + dcdq * (f_area + f_damp);
    f2 = f2 + dcdr * (f_area + f_damp);
    V3<S> f0 = f1 + f2;
    const V3<S> vmid = (v[0] + v[1] + v[2]) * 0.3333f;
    const V3<S> vdir = gnormalize(vmid);
    const V3<S> f_drag = vmid * (area * k_drag * gabs(gdot(n, vmid)));
    const V3<S> f_lift = n * (area * k_lift * (1.57079632679489661923f - gacos(gdot(n, vdir)))) * gdot(vmid, vmid);
    f0 = f0 - f_drag - f_lift;
    f1 = f1 + f_drag + f_lift;
    f2 = f2 + f_drag + f_lift;
    out[0] = f0;
    out[1] = -f1;
    out[2] = -f2;
}

// Bend-torque force of one spring (added to node j, subtracted from node i)
// from xij = x_i - x_j and vij = v_i - v_j, toward the rest direction
// d0 = -rest_direction.  Returns false where the reference skips the torque
// (|d0| < 0.5, |xij| < 1e-6 or a vanishing rotation axis).  Reference
// kernels.py:221-291.
template <class S>
__device__ __forceinline__ bool spring_torque_force(V3<S> xij, V3<S> vij, float3 rest_direction, float kt, float kwt,
                                                    V3<S>& out) {
    const float3 d0f = make_float3(-rest_direction.x, -rest_direction.y, -rest_direction.z);
    if (sqrtf(d0f.x * d0f.x + d0f.y * d0f.y + d0f.z * d0f.z) < 0.5f) return false;
    const S L = glength(xij);
    if (val(L) < 1.0e-6f) return false;
    const V3<S> d = xij / L;
    const V3<S> d0 = lift3<S>(d0f);
    const S theta = gacos(gclamp(gdot(d, d0), -1.0f, 1.0f));
    V3<S> axis = gcross(d0, d);
    const S axis_len = glength(axis);
    if (val(axis_len) < 1.0e-6f) return false;
    axis = axis / axis_len;
    const V3<S> d_dot = (vij - d * gdot(d, vij)) / L;
    const S omega = gdot(gcross(d, d_dot), axis);
    const S tau = -(theta * kt + omega * kwt) * L;
    out = gcross(axis * tau, d) / L;
    return true;
}

}  // namespace fem
