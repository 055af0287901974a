// Element and node kernels of the FEM hot path (sm_103a):
//   node_prepare      fixed-node restore + float4 packing of q, v and the CG warm start
//   tet_force         Stable Neo-Hookean Tet4 force + Rayleigh damping (+ activation), per element
//   hex_force         Q1 Hex8 force, 8 lanes per element (one per Gauss point)
//   tri_force         triangle membrane + area + drag/lift force, per element
//   node_forces       deterministic element->node gather + springs (with bend torque), particle
//                     and soft contacts, ground, gravity, damping, and the h-scaled sum in the
//                     reference's term order
//   constant_blocks   mass + spring diagonal, spring off-diagonal and lumped triangle blocks
//   tet_tangent       16 PSD blocks per tet (per-tet factors staged in shared memory)
//   hex_tangent       64 PSD blocks per hex (Gauss-point data computed once per element)
// No float atomics anywhere: every sum runs in a fixed order.
#include <climits>

#include "fem_generic.cuh"
#include "fem_internal.cuh"
#include "fem_math.cuh"

namespace fem {

__constant__ float c_dNdxi[8][8][3];  // [gauss point][node][d/dxi, d/deta, d/dzeta]

namespace {

__device__ __forceinline__ float3 load3(const float* p, int i) { return f3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ void store3(float* p, int i, float3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}

__global__ void node_prepare_kernel(int P, float* __restrict__ q, float* __restrict__ v,
                                    const unsigned char* __restrict__ fixed_mask, const float* __restrict__ rest,
                                    const float* __restrict__ dv, float4* __restrict__ q4, float4* __restrict__ v4,
                                    float4* __restrict__ x4, int restore, int pack_v, int pack_x) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    bool fx = fixed_mask[i] != 0;
    if (!restore) {  // plain packing, caller arrays untouched
        q4[i] = f4(load3(q, i));
        if (pack_v) v4[i] = f4(load3(v, i));
        if (pack_x) x4[i] = fx ? make_float4(0.f, 0.f, 0.f, 0.f) : f4(load3(dv, i));
        return;
    }
    float3 qi;
    if (fx) {  // fixed_particles.py:11-21 restore q (and v) in place
        qi = load3(rest, i);
        store3(q, i, qi);
    } else {
        qi = load3(q, i);
    }
    q4[i] = f4(qi);
    if (pack_v) {
        float3 vi = f3(0.f, 0.f, 0.f);
        if (fx) store3(v, i, vi);
        else vi = load3(v, i);
        v4[i] = f4(vi);
    }
    if (pack_x) x4[i] = fx ? make_float4(0.f, 0.f, 0.f, 0.f) : f4(load3(dv, i));
}

// Reference kernels.py:511-632 (force) and 484-508 (activation).  Writes the
// restoring force of each corner into out[4 t + a].
__global__ void __launch_bounds__(128, 8) tet_force_kernel(int T, const int4* __restrict__ idx, const float* __restrict__ pose,
                                 const float* __restrict__ mat, const float4* __restrict__ q4,
                                 const float4* __restrict__ v4, const float* __restrict__ act,
                                 const float* __restrict__ mu_scale, float lo, float hi, float4* __restrict__ out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    int4 n = idx[t];
    float k_mu = mat[3 * t], k_lambda = mat[3 * t + 1], k_damp = mat[3 * t + 2];
    if (mu_scale != nullptr) k_mu *= mu_scale[t];  // per-element shear scale (differentiable control)
    float4* o = out + 4 * t;
    if (k_mu == 0.0f && k_lambda == 0.0f && k_damp == 0.0f) {
        float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        o[0] = zero; o[1] = zero; o[2] = zero; o[3] = zero;
        return;
    }
    float3 x0 = xyz(q4[n.x]), x1 = xyz(q4[n.y]), x2 = xyz(q4[n.z]), x3 = xyz(q4[n.w]);
    float3 v0 = xyz(v4[n.x]), v1 = xyz(v4[n.y]), v2 = xyz(v4[n.z]), v3 = xyz(v4[n.w]);
    float3 x10 = x1 - x0, x20 = x2 - x0, x30 = x3 - x0;
    float3 v10 = v1 - v0, v20 = v2 - v0, v30 = v3 - v0;
    M3 Dm;
#pragma unroll
    for (int k = 0; k < 9; ++k) Dm.m[k / 3][k % 3] = pose[9 * t + k];
    float inv_rest_volume = det3(Dm) * 6.0f;
    float rest_volume = 1.0f / inv_rest_volume;
    float alpha = 1.0f + k_mu / k_lambda - k_mu / (4.0f * k_lambda);
    float mu = k_mu * rest_volume, lam = k_lambda * rest_volume, damp = k_damp * rest_volume;
    M3 F = clamp_stretch(matmul(from_cols(x10, x20, x30), Dm), lo, hi);
    M3 dFdt = matmul(from_cols(v10, v20, v30), Dm);
    float3 c0 = col(F, 0), c1 = col(F, 1), c2 = col(F, 2);
    float Ic = dot3(c0, c0) + dot3(c1, c1) + dot3(c2, c2);
    float sdev = mu * (1.0f - 1.0f / (Ic + 1.0f));
    M3 P;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) P.m[i][j] = F.m[i][j] * sdev + dFdt.m[i][j] * damp;
    M3 Hm = matmulT(P, Dm);
    float3 f1 = col(Hm, 0), f2 = col(Hm, 1), f3v = col(Hm, 2);
    float J = fmaxf(det3(F), 0.01f);
    float s = inv_rest_volume / 6.0f;
    float3 d1 = cross3(x20, x30) * s, d2 = cross3(x30, x10) * s, d3 = cross3(x10, x20) * s;
    float f_volume = (J - alpha) * lam;
    float f_damp = (dot3(d1, v10) + dot3(d2, v20) + dot3(d3, v30)) * damp;
    float ft = f_volume + f_damp;
    f1 = f1 + d1 * ft;
    f2 = f2 + d2 * ft;
    f3v = f3v + d3 * ft;
    float3 f0 = -(f1 + f2 + f3v);
    // restoring force = -f_a (the reference subtracts f_a from the buffer)
    float3 r0 = -f0, r1 = -f1, r2 = -f2, r3 = -f3v;
    if (act != nullptr) {
        float sc = k_lambda * act[t] / 6.0f;
        float3 fb = cross3(x2 - x0, x3 - x0) * sc;
        float3 fc = cross3(x3 - x0, x1 - x0) * sc;
        float3 fd = cross3(x1 - x0, x2 - x0) * sc;
        r0 = r0 + (fb + fc + fd);
        r1 = r1 - fb;
        r2 = r2 - fc;
        r3 = r3 - fd;
    }
    o[0] = f4(r0);
    o[1] = f4(r1);
    o[2] = f4(r2);
    o[3] = f4(r3);
}

// Walsh-Hadamard transform over the 8 lanes of a hex group: lane m ends with
// sum_a chi_m(a) v_a, chi_m(a) = (-1)^popcount(a & m), v_a the value of lane a.
__device__ __forceinline__ float wht8(float v, int lane8) {
#pragma unroll
    for (int b = 1; b < 8; b <<= 1) {
        const float o = __shfl_xor_sync(0xffffffffu, v, b);
        v = (lane8 & b) ? o - v : v + o;
    }
    return v;
}

// Reference kernels.py:1481-1601.  Lane g of an 8-lane group evaluates Gauss point g of one hex,
// lane a holds node a.  In VTK order node a has the signs s_x = (a0 xor a1) ? +1 : -1,
// s_y = a1 ? +1 : -1, s_z = a2 ? +1 : -1 (a0..a2 its bits), and the trilinear shape functions give
//   dx/dxi = (c_x + eta c_xy + zeta c_xz + eta zeta c_xyz) / 8 (likewise for eta, zeta),
// c_S = sum_a (prod_{s in S} s(a)) x_a.  Those sums are Walsh-Hadamard coefficients of the node
// values over the lanes (c_x = -H3, c_y = -H2, c_z = -H4, c_xy = H1, c_xz = H7, c_yz = H6,
// c_xyz = -H5), so F = (dx/dxi) inv_J0 and dF/dt come from one 3-stage butterfly and 7 broadcasts
// per component instead of an 8-node sum per entry.  The corner forces f_a = sum_g (P inv_J0^T w)_g
// dN_a/dxi(g) use the same identity the other way: a butterfly of the points' P inv_J0^T w gives
// the sums over points weighted by 1, xi, eta, zeta and their products, from which lane a forms its
// corner force.
__global__ void __launch_bounds__(256, 4) hex_force_kernel(int H, const int* __restrict__ idx,
                                                        const float* __restrict__ invJ,
                                                        const float* __restrict__ detw,
                                                        const float* __restrict__ mat,
                                                        const float4* __restrict__ q4,
                                                        const float4* __restrict__ v4, float lo, float hi,
                                                        float4* __restrict__ out) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int h = gid >> 3, g = gid & 7;
    const bool live = h < H;
    const int64_t he = live ? h : H - 1;  // lanes past the end work on a valid hex and store nothing
    const int node = idx[8 * he + g];
    const float4 xg = q4[node], vg = v4[node];
    const float k_mu = mat[3 * he], k_lambda = mat[3 * he + 1], k_damp = mat[3 * he + 2];
    const float alpha = 1.0f + k_mu / k_lambda - k_mu / (4.0f * k_lambda);
    M3 iJ;
#pragma unroll
    for (int k = 0; k < 9; ++k) iJ.m[k / 3][k % 3] = invJ[(8 * he + g) * 9 + k] * 0.125f;  // the 1/8, exactly
    const float w = detw[8 * he + g];
    const int base = threadIdx.x & 24;  // first lane of this 8-lane group within the warp
    // this lane's point (and, later, node) signs and Gauss coordinates
    const float sx = ((g ^ (g >> 1)) & 1) ? 1.0f : -1.0f, sy = (g & 2) ? 1.0f : -1.0f, sz = (g & 4) ? 1.0f : -1.0f;
    const float gp = 0.5773502691896258f;
    const float xi = sx * gp, eta = sy * gp, zeta = sz * gp;
    const float ez = eta * zeta, xz = xi * zeta, xe = xi * eta;
    // (dx/dxi) for positions and velocities: columns (d/dxi, d/deta, d/dzeta)
    M3 GX, GV;
#pragma unroll
    for (int f = 0; f < 2; ++f) {
        const float4 src = f == 0 ? xg : vg;
        const float comp[3] = {src.x, src.y, src.z};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float t = wht8(comp[i], g);
            const float h1 = __shfl_sync(0xffffffffu, t, base + 1), h2 = __shfl_sync(0xffffffffu, t, base + 2);
            const float h3 = __shfl_sync(0xffffffffu, t, base + 3), h4 = __shfl_sync(0xffffffffu, t, base + 4);
            const float h5 = __shfl_sync(0xffffffffu, t, base + 5), h6 = __shfl_sync(0xffffffffu, t, base + 6);
            const float h7 = __shfl_sync(0xffffffffu, t, base + 7);
            const float d0 = fmaf(-ez, h5, fmaf(zeta, h7, fmaf(eta, h1, -h3)));
            const float d1 = fmaf(-xz, h5, fmaf(zeta, h6, fmaf(xi, h1, -h2)));
            const float d2 = fmaf(-xe, h5, fmaf(eta, h6, fmaf(xi, h7, -h4)));
            M3& G = f == 0 ? GX : GV;
            G.m[i][0] = d0;
            G.m[i][1] = d1;
            G.m[i][2] = d2;
        }
    }
    M3 F = matmul(GX, iJ);
    const M3 dFdt = matmul(GV, iJ);
    F = clamp_stretch(F, lo, hi);
    const float3 fc0 = col(F, 0), fc1 = col(F, 1), fc2 = col(F, 2);
    const float Ic = dot3(fc0, fc0) + dot3(fc1, fc1) + dot3(fc2, fc2);
    const float sdev = k_mu * (1.0f - 1.0f / (Ic + 1.0f));
    const float J = fmaxf(det3(F), 0.01f);
    const M3 cof = from_cols(cross3(fc1, fc2), cross3(fc2, fc0), cross3(fc0, fc1));
    const float vol = k_lambda * (J - alpha);
    M3 P;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) P.m[i][j] = ((F.m[i][j] * sdev + dFdt.m[i][j] * k_damp) + cof.m[i][j] * vol) * w;
    // P inv_J0^T w with the 1/8 of the shape-function derivatives (carried by the scaled inv_J0)
    const M3 PJ = matmulT(P, iJ);
    // node a = g: f_a[i] = s_x (W0 + s_y Se + s_z Sz + s_y s_z Sez)[i][0]
    //                    + s_y (W0 + s_x Sx + s_z Sz + s_x s_z Sxz)[i][1]
    //                    + s_z (W0 + s_x Sx + s_y Se + s_x s_y Sxe)[i][2],
    // with Sx = -gp W3, Se = -gp W2, Sz = -gp W4, Sez = gp^2 W6, Sxz = gp^2 W7, Sxe = gp^2 W1 and
    // W_m = sum_g chi_m(g) PJ_g (the butterfly below)
    const float gp2 = gp * gp;
    const float cy = -gp * sy, cz = -gp * sz, cx = -gp * sx;
    const float cyz = gp2 * sy * sz, cxz = gp2 * sx * sz, cxy = gp2 * sx * sy;
    float fa[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float w0 = wht8(PJ.m[i][0], g), w1 = wht8(PJ.m[i][1], g), w2 = wht8(PJ.m[i][2], g);
        const float a00 = __shfl_sync(0xffffffffu, w0, base), a01 = __shfl_sync(0xffffffffu, w1, base);
        const float a02 = __shfl_sync(0xffffffffu, w2, base);
        const float e20 = __shfl_sync(0xffffffffu, w0, base + 2), e22 = __shfl_sync(0xffffffffu, w2, base + 2);
        const float z40 = __shfl_sync(0xffffffffu, w0, base + 4), z41 = __shfl_sync(0xffffffffu, w1, base + 4);
        const float ez60 = __shfl_sync(0xffffffffu, w0, base + 6);
        const float x31 = __shfl_sync(0xffffffffu, w1, base + 3), x32 = __shfl_sync(0xffffffffu, w2, base + 3);
        const float xz71 = __shfl_sync(0xffffffffu, w1, base + 7);
        const float xe12 = __shfl_sync(0xffffffffu, w2, base + 1);
        const float t0 = fmaf(cyz, ez60, fmaf(cz, z40, fmaf(cy, e20, a00)));
        const float t1 = fmaf(cxz, xz71, fmaf(cz, z41, fmaf(cx, x31, a01)));
        const float t2 = fmaf(cxy, xe12, fmaf(cy, e22, fmaf(cx, x32, a02)));
        fa[i] = fmaf(sz, t2, fmaf(sy, t1, sx * t0));
    }
    if (live) out[8 * h + g] = make_float4(-fa[0], -fa[1], -fa[2], 0.0f);
}

// Reference kernels.py:876-960: one thread per triangle writes its three
// corner forces to the element-force slots 3e..3e+2 (after the Tet4/Hex8 slots).
__global__ void tri_force_kernel(int Tri, const int* __restrict__ idx, const float4* __restrict__ pose,
                                 const float* __restrict__ mat, const float4* __restrict__ q4,
                                 const float4* __restrict__ v4, float4* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= Tri) return;
    V3<float> x[3], v[3], f[3];
    float m[5];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int n = idx[3 * e + c];
        const float4 qn = q4[n], vn = v4[n];
        x[c] = v3(qn.x, qn.y, qn.z);
        v[c] = v3(vn.x, vn.y, vn.z);
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) m[k] = mat[5 * e + k];
    triangle_force(x, v, pose[e], m, f);
#pragma unroll
    for (int c = 0; c < 3; ++c) out[3 * e + c] = make_float4(f[c].x, f[c].y, f[c].z, 0.0f);
}

struct NodeForceArgs {
    int P, T, H;
    const float4* q4;
    const float4* v4;
    const int* elem_ptr;
    const int* elem_ent;
    const float4* elem_force;
    const int* spring_ptr;
    const int* spring_ent;
    const int* spring_idx;
    const float* spring_rest;
    const float* spring_ke;
    const float* spring_kd;
    const float* spring_dir;  // rest directions when the bend torque is active
    float torque_ke, torque_kd;
    const float4* pforce;     // particle-contact force per node, or null
    const int* sc_head;       // soft-contact list per node, or null
    const int* sc_next;
    const float4* sc_force;
    const float4* sforce;     // surface-contact force per node, or null
    const float* mass;
    const float* inv_mass;
    const float* radius;
    const int* flags;
    const float* gravity;
    const float* ext;
    float ground[4];
    float gke, gkd, gkf, gmu;
    int has_ground;
    float linear_damping;
    float dt;
    int terms;
    int scale_by_dt;
    float* out;
};

// Reference solver.py:542-589 (term order), kernels.py:176-218 (springs),
// 221-291 (bend torque), 1132-1195 (ground), 1198-1261 (soft contacts),
// 1273-1307 (gravity, damping), soft_surface_contacts.py (surface).  Term
// order: spring, tet, hex, tri, particle, ground, soft contact, gravity,
// damping, surface.
// kFull = false compiles out the spring (and bend torque) and contact terms, for scenes that have
// none: the remaining gather then fits in fewer registers, so more warps cover its load latency.
template <bool kFull>
__global__ void node_forces_kernel(NodeForceArgs a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.P) return;
    float3 xi = xyz(a.q4[i]), vi = xyz(a.v4[i]);
    float3 zero = f3(0.f, 0.f, 0.f);
    float3 fs = zero, ft = zero, fh = zero, ftri = zero, fp = zero, fg = zero, fsc = zero, fgr = zero, fd = zero,
           fsf = zero;
    // The incident springs and element corners are read kSpringBatch /
    // kCornerBatch at a time (ids, then the data they index) before any is
    // added, so that many independent loads are in flight; the sums keep the
    // ascending incidence order.
    if (kFull && (a.terms & FEM_TERM_SPRING)) {
        constexpr int kSpringBatch = 2;
        const int e1 = a.spring_ptr[i + 1];
        for (int e0 = a.spring_ptr[i]; e0 < e1; e0 += kSpringBatch) {
            int ent[kSpringBatch], ia[kSpringBatch], ib[kSpringBatch];
#pragma unroll
            for (int u = 0; u < kSpringBatch; ++u) ent[u] = e0 + u < e1 ? __ldg(a.spring_ent + e0 + u) : -1;
#pragma unroll
            for (int u = 0; u < kSpringBatch; ++u) {
                const int sp = ent[u] < 0 ? 0 : ent[u] >> 1;
                ia[u] = ent[u] < 0 ? -1 : __ldg(a.spring_idx + 2 * sp);
                ib[u] = ent[u] < 0 ? -1 : __ldg(a.spring_idx + 2 * sp + 1);
            }
            float3 xij[kSpringBatch], vij[kSpringBatch];
            float rest[kSpringBatch], ke[kSpringBatch], kd[kSpringBatch];
#pragma unroll
            for (int u = 0; u < kSpringBatch; ++u) {
                const bool ok = ia[u] >= 0 && ib[u] >= 0;
                const int ja = ok ? ia[u] : 0, jb = ok ? ib[u] : 0, sp = ok ? ent[u] >> 1 : 0;
                xij[u] = xyz(a.q4[ja]) - xyz(a.q4[jb]);
                vij[u] = xyz(a.v4[ja]) - xyz(a.v4[jb]);
                rest[u] = a.spring_rest[sp];
                ke[u] = a.spring_ke[sp];
                kd[u] = a.spring_kd[sp];
            }
#pragma unroll
            for (int u = 0; u < kSpringBatch; ++u) {
                if (ia[u] < 0 || ib[u] < 0) continue;
                const float L = len3(xij[u]);
                if (L < 1.0e-6f) continue;
                const float3 dir = f3(xij[u].x / L, xij[u].y / L, xij[u].z / L);
                const float c = L - rest[u];
                const float dcdt = dot3(dir, vij[u]);
                const float3 f = dir * (ke[u] * c + kd[u] * dcdt);
                fs = (ent[u] & 1) ? fs + f : fs - f;
                if (a.spring_dir != nullptr) {  // kernels.py:266-291
                    const int sp = ent[u] >> 1;
                    const float3 d0 = f3(a.spring_dir[3 * sp], a.spring_dir[3 * sp + 1], a.spring_dir[3 * sp + 2]);
                    V3<float> tq;
                    if (spring_torque_force(v3(xij[u].x, xij[u].y, xij[u].z), v3(vij[u].x, vij[u].y, vij[u].z), d0,
                                            a.torque_ke, a.torque_kd, tq))
                        fs = (ent[u] & 1) ? fs + f3(tq.x, tq.y, tq.z) : fs - f3(tq.x, tq.y, tq.z);
                }
            }
        }
    }
    if (a.terms & (FEM_TERM_TET | FEM_TERM_HEX | FEM_TERM_TRI)) {
        constexpr int kCornerBatch = 8;
        const int tet_end = 4 * a.T, hex_end = 4 * a.T + 8 * a.H;
        const int e1 = a.elem_ptr[i + 1];
        for (int e0 = a.elem_ptr[i]; e0 < e1; e0 += kCornerBatch) {
            int ent[kCornerBatch];
            float3 f[kCornerBatch];
#pragma unroll
            for (int u = 0; u < kCornerBatch; ++u) ent[u] = e0 + u < e1 ? __ldg(a.elem_ent + e0 + u) : -1;
#pragma unroll
            for (int u = 0; u < kCornerBatch; ++u) f[u] = xyz(a.elem_force[ent[u] < 0 ? 0 : ent[u]]);
#pragma unroll
            for (int u = 0; u < kCornerBatch; ++u) {
                if (ent[u] < 0) continue;
                if (ent[u] < tet_end) {
                    if (a.terms & FEM_TERM_TET) ft = ft + f[u];
                } else if (ent[u] < hex_end) {
                    if (a.terms & FEM_TERM_HEX) fh = fh + f[u];
                } else if (a.terms & FEM_TERM_TRI) {
                    ftri = ftri + f[u];
                }
            }
        }
    }
    if (kFull && (a.terms & FEM_TERM_PARTICLE) && a.pforce != nullptr) fp = xyz(a.pforce[i]);
    bool active = (a.flags[i] & 1) != 0;
    float3 grav = f3(a.gravity[0], a.gravity[1], a.gravity[2]);
    if ((a.terms & FEM_TERM_GROUND) && a.has_ground && active) {
        float3 n = f3(a.ground[0], a.ground[1], a.ground[2]);
        float c = fminf(dot3(n, xi) + a.ground[3] - a.radius[i], 0.0f);
        if (c < 0.0f) {
            float vn = dot3(n, vi);
            float jn = c * a.gke;
            float jd = fminf(vn, 0.0f) * a.gkd;
            float fn = jn + jd;
            float3 vt = vi - n * vn;
            float vs = len3(vt);
            if (vs > 0.0f) vt = f3(vt.x / vs, vt.y / vs, vt.z / vs);
            float gmag = len3(grav);
            float inv_m = a.inv_mass[i];
            float inv_m_safe = fmaxf(inv_m, 1e-9f);
            float m = inv_m > 0.0f ? 1.0f / inv_m_safe : 0.0f;
            float fn_eff = fminf(fabsf(fn), m * gmag);
            float ftan = fminf(vs * a.gkf, a.gmu * fn_eff);
            fg = zero - n * fn - vt * ftan;
        }
    }
    if (kFull && (a.terms & FEM_TERM_SOFT_CONTACT) && a.sc_head != nullptr) {
        // the list holds this node's penetrating contacts in arbitrary order: add
        // them in ascending contact id (repeated minimum search, lists are short)
        int last = -1;
        for (;;) {
            int next = INT_MAX;
            for (int c = a.sc_head[i]; c >= 0; c = a.sc_next[c])
                if (c > last && c < next) next = c;
            if (next == INT_MAX) break;
            fsc = fsc + xyz(a.sc_force[next]);
            last = next;
        }
    }
    if ((a.terms & FEM_TERM_GRAVITY) && active) {
        float m = a.mass[i];
        fgr = f3(grav.x * m, grav.y * m, grav.z * m);
    }
    if ((a.terms & FEM_TERM_DAMPING) && active && a.linear_damping > 0.0f) {
        fd = vi * (-a.linear_damping * a.mass[i]);
    }
    if (kFull && (a.terms & FEM_TERM_SURFACE) && a.sforce != nullptr) fsf = xyz(a.sforce[i]);
    float3 f;
    if (a.scale_by_dt) {
        float h = a.dt;
        f = fs * h;
        f = f + ft * h;
        f = f + fh * h;
        f = f + ftri * h;
        f = f + fp * h;
        f = f + fg * h;
        f = f + fsc * h;
        f = f + fgr * h;
        f = f + fd * h;
        f = f + fsf * h;
        if (a.ext != nullptr) f = f + load3(a.ext, i) * h;
    } else {
        f = fs + ft + fh + ftri + fp + fg + fsc + fgr + fd + fsf;
    }
    store3(a.out, i, f);
}

// Reference kernels.py:294-323 (diagonal with springs), 141-153 (mass only), 326-366 (off-diagonal).
__global__ void constant_diag_kernel(int P, const float* __restrict__ mass, const int* __restrict__ sptr,
                                     const int* __restrict__ sent, const float* __restrict__ ke,
                                     const float* __restrict__ kd, float dt, TripletPlanes vals) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    float dt2 = dt * dt;
    float d = mass[i];
    for (int e = sptr[i]; e < sptr[i + 1]; ++e) {
        int s = sent[e] >> 1;
        d = d + dt * kd[s] + dt2 * ke[s];
    }
    const float o[9] = {d, 0.f, 0.f, 0.f, d, 0.f, 0.f, 0.f, d};
    store_block(vals, i, o);
}

__global__ void constant_offdiag_kernel(int P, int S, const float* __restrict__ ke, const float* __restrict__ kd,
                                        float dt, TripletPlanes vals) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    float neg_off = -(dt * kd[s] + dt * dt * ke[s]);
    const float o[9] = {neg_off, 0.f, 0.f, 0.f, neg_off, 0.f, 0.f, 0.f, neg_off};
    for (int k = 0; k < 2; ++k) store_block(vals, (int64_t)P + 2 * (int64_t)s + k, o);
}

// Reference kernels.py:963-1012: h^2 (mu + lambda) A_rest / 3 on each vertex's
// diagonal (zero blocks for a degenerate rest triangle), position independent.
__global__ void constant_tri_kernel(int Tri, const float4* __restrict__ pose, const float* __restrict__ mat, float dt,
                                    int64_t trip_off, TripletPlanes vals) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= Tri) return;
    const float4 Dm = pose[e];
    const float inv_rest_area = (Dm.x * Dm.w - Dm.y * Dm.z) * 2.0f;
    float d = 0.0f;
    if (inv_rest_area > 0.0f) {
        const float rest_area = 1.0f / inv_rest_area;
        d = dt * dt * (mat[5 * e] * rest_area + mat[5 * e + 1] * rest_area) / 3.0f;
    }
    const float o[9] = {d, 0.f, 0.f, 0.f, d, 0.f, 0.f, 0.f, d};
    for (int c = 0; c < 3; ++c) store_block(vals, trip_off + 3 * (int64_t)e + c, o);
}

constexpr int kTetTangentThreads = 128;
constexpr int kTetFactor = 40;

// Reference kernels.py:635-850.  Phase 1: one thread per tet computes the
// per-tet factors (F dm_a, dJ/dx_a, dm_a and three coefficients) into shared
// memory.  Phase 2: 16 consecutive threads write the 16 blocks of a tet, so
// the 576-byte block run of each element is written contiguously.
__global__ void __launch_bounds__(kTetTangentThreads) tet_tangent_kernel(
    int T, const int4* __restrict__ idx, const float* __restrict__ pose, const float* __restrict__ mat,
    const float* __restrict__ mu_scale, const float4* __restrict__ q4, float lo, float hi, float dt, int64_t trip_off,
    TripletPlanes vals) {
    __shared__ float sm[kTetTangentThreads][kTetFactor + 1];
    int lt = threadIdx.x;
    int t = blockIdx.x * kTetTangentThreads + lt;
    float* fct = sm[lt];
    if (t < T) {
        float k_mu = mat[3 * t], k_lambda = mat[3 * t + 1];
        if (mu_scale != nullptr) k_mu *= mu_scale[t];
        if (k_mu == 0.0f && k_lambda == 0.0f && mat[3 * t + 2] == 0.0f) {
            fct[39] = 2.0f;  // empty material: rows/cols are -1, nothing to write
        } else {
            M3 Dm;
#pragma unroll
            for (int k = 0; k < 9; ++k) Dm.m[k / 3][k % 3] = pose[9 * t + k];
            float inv_rest_volume = det3(Dm) * 6.0f;
            if (inv_rest_volume <= 0.0f) {
                fct[39] = 1.0f;  // degenerate rest pose: zero blocks at valid rows
            } else {
                int4 n = idx[t];
                float3 x0 = xyz(q4[n.x]), x1 = xyz(q4[n.y]), x2 = xyz(q4[n.z]), x3 = xyz(q4[n.w]);
                float3 x10 = x1 - x0, x20 = x2 - x0, x30 = x3 - x0;
                float rest_volume = 1.0f / inv_rest_volume;
                float mu = k_mu * rest_volume, lam = k_lambda * rest_volume;
                M3 F = clamp_stretch(matmul(from_cols(x10, x20, x30), Dm), lo, hi);
                float3 c0 = col(F, 0), c1 = col(F, 1), c2 = col(F, 2);
                float Ic = dot3(c0, c0) + dot3(c1, c1) + dot3(c2, c2);
                float Ic1 = fmaxf(Ic + 1.0f, 1e-6f);
                float s = 1.0f - 1.0f / Ic1;
                float coef = mu * 2.0f / (Ic1 * Ic1);
                float sv = inv_rest_volume / 6.0f;
                float3 d1 = cross3(x20, x30) * sv, d2 = cross3(x30, x10) * sv, d3 = cross3(x10, x20) * sv;
                float3 d0 = -(d1 + d2 + d3);
                float3 m1 = row(Dm, 0), m2 = row(Dm, 1), m3 = row(Dm, 2);
                float3 m0 = -(m1 + m2 + m3);
                float3 dJ[4] = {d0, d1, d2, d3};
                float3 dm[4] = {m0, m1, m2, m3};
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    float3 fd = mul(F, dm[a]);
                    fct[3 * a] = fd.x; fct[3 * a + 1] = fd.y; fct[3 * a + 2] = fd.z;
                    fct[12 + 3 * a] = dJ[a].x; fct[13 + 3 * a] = dJ[a].y; fct[14 + 3 * a] = dJ[a].z;
                    fct[24 + 3 * a] = dm[a].x; fct[25 + 3 * a] = dm[a].y; fct[26 + 3 * a] = dm[a].z;
                }
                fct[36] = mu * s;
                fct[37] = coef;
                fct[38] = lam;
                fct[39] = 0.0f;
            }
        }
    }
    __syncthreads();
    float scale = dt * dt;
#pragma unroll 4
    for (int m = 0; m < 16; ++m) {
        int b = lt + kTetTangentThreads * m;
        int le = b >> 4, ab = b & 15;
        int te = blockIdx.x * kTetTangentThreads + le;
        if (te >= T) continue;
        const float* f = sm[le];
        float mode = f[39];
        if (mode == 2.0f) continue;
        const int64_t ti = trip_off + 16 * (int64_t)te + ab;
        float o[9];
        if (mode == 1.0f) {
#pragma unroll
            for (int k = 0; k < 9; ++k) o[k] = 0.0f;
            store_block(vals, ti, o);
            continue;
        }
        int a = ab >> 2, bb = ab & 3;
        float3 Fa = f3(f[3 * a], f[3 * a + 1], f[3 * a + 2]);
        float3 Fb = f3(f[3 * bb], f[3 * bb + 1], f[3 * bb + 2]);
        float3 Ja = f3(f[12 + 3 * a], f[13 + 3 * a], f[14 + 3 * a]);
        float3 Jb = f3(f[12 + 3 * bb], f[13 + 3 * bb], f[14 + 3 * bb]);
        float3 ma = f3(f[24 + 3 * a], f[25 + 3 * a], f[26 + 3 * a]);
        float3 mb = f3(f[24 + 3 * bb], f[25 + 3 * bb], f[26 + 3 * bb]);
        float diag = f[36] * dot3(ma, mb);
        float coef = f[37], lam = f[38];
        float fa[3] = {Fa.x, Fa.y, Fa.z}, fb[3] = {Fb.x, Fb.y, Fb.z};
        float ja[3] = {Ja.x, Ja.y, Ja.z}, jb[3] = {Jb.x, Jb.y, Jb.z};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                float kdev = (i == j ? diag : 0.0f) + fa[i] * fb[j] * coef;
                float kvol = ja[i] * jb[j] * lam;
                o[3 * i + j] = (kdev + kvol) * scale;
            }
        store_block(vals, ti, o);
    }
}

// Hex8 tangent (reference kernels.py:1609-1747):
//   K_ab = h^2 sum_g [c1 (gN_a . gN_b) I + c2 (F gN_a)(F gN_b)^T + c3 (cof F gN_a)(cof F gN_b)^T],
// c1 = k_mu s w_g, c2 = 2 k_mu w_g / (Ic + 1)^2, c3 = k_lambda w_g, with F, the stretch clamp and
// cof F formed once per Gauss point.  Every term is an outer product of per-(point, node) vectors,
// so with r = h (sqrt|c1| gN_a, sqrt|c2| F gN_a, sqrt|c3| cof F gN_a) the block is
//   K_ab = sum_g [(r1_a . r1_b) I + r2_a r2_b^T + r3_a r3_b^T]   (signs of c applied when negative).
// A CTA takes kTanHex hexes:
//   phase 0  the hexes' node positions and the Gauss table are staged in shared memory, and the
//            phase-1 threads load their point's inverse Jacobian, weight and materials, so every
//            global load of the CTA is in flight before the first barrier;
//   phase 1  one thread per (hex, point) forms gN_a, F, the clamp, cof F and the eight 9-float
//            records r of its point (no work repeated across lanes);
//   phase 2  one thread per 2x2 tile of blocks on or above the block diagonal (10 tiles per
//            hex) sums its four blocks over the 8 points; a tile off the diagonal also gives
//            the four transposed blocks below it (K_ba = K_ab^T term by term, so A is
//            exactly symmetric).  Threads are tile-major (16 hexes per tile), so a quarter
//            warp reads 8 hexes' records in 8 distinct bank groups and a diagonal tile's half
//            warp skips its column-side loads;
//   phase 3  the 64 blocks per hex are staged in shared memory in the triplet planes' layout
//            (hexes padded apart so the staging stores are conflict-free) and written out by
//            bulk asynchronous copies (cp.async.bulk), one per hex and plane.
constexpr int kTanHex = 16;
constexpr int kTanTiles = 10;
constexpr int kTanThreads = kTanHex * kTanTiles;
constexpr int kTanRec = 12;                                // words per record (9 used)
constexpr int kTanPointStride = 8 * kTanRec + 4;           // padded: the 8 points of a hex in distinct banks
constexpr int kTanHexStride = 8 * kTanPointStride + 4;     // padded: hexes of a warp in distinct banks
constexpr int kTanTabStride = 28;                          // padded Gauss table row
constexpr int kTanSgnStride = 9;                           // padded per-hex row of point signs
constexpr int kTanOut4Stride = 65;                         // staged float4 blocks per hex (padded)
constexpr int kTanOut1Stride = 68;                         // staged last-entry floats per hex (padded)
constexpr size_t kTanRecBytes = sizeof(float) * kTanHex * kTanHexStride;
constexpr size_t kTanOutA = 0, kTanOutB = 16 * kTanOut4Stride * kTanHex, kTanOutC = 2 * kTanOutB;
constexpr size_t kTanXOff = kTanRecBytes;
constexpr size_t kTanSgnOff = kTanXOff + 16 * 8 * kTanHex;
constexpr size_t kTanTabOff = kTanSgnOff + 16 * kTanSgnStride * kTanHex;
constexpr size_t kTanSmemBytes = kTanTabOff + sizeof(float) * 8 * kTanTabStride;
static_assert(kTanOutC + 4 * kTanOut1Stride * kTanHex <= kTanRecBytes, "output staging reuses the record area");
static_assert((16 * kTanOut4Stride) % 16 == 0 && (4 * kTanOut1Stride) % 16 == 0, "16-byte bulk copy sources");
static_assert(kTanRec % 4 == 0 && kTanPointStride % 4 == 0 && kTanHexStride % 4 == 0, "16-byte records");

__device__ __forceinline__ void tan_tile_rows(int t, int& A, int& B) {
    // (0,0) (0,1) (0,2) (0,3) (1,1) (1,2) (1,3) (2,2) (2,3) (3,3)
    A = t < 4 ? 0 : (t < 7 ? 1 : (t < 9 ? 2 : 3));
    B = A + t - (A == 0 ? 0 : (A == 1 ? 4 : (A == 2 ? 7 : 9)));
}

__device__ __forceinline__ void tan_load_record(const float* p, float (&r)[9]) {
    const float4 v0 = reinterpret_cast<const float4*>(p)[0];
    const float4 v1 = reinterpret_cast<const float4*>(p)[1];
    r[0] = v0.x; r[1] = v0.y; r[2] = v0.z; r[3] = v0.w;
    r[4] = v1.x; r[5] = v1.y; r[6] = v1.z; r[7] = v1.w;
    r[8] = p[8];
}

// The four blocks (a0 + i, b0 + j) of one tile, summed over the 8 points in order; kSigned applies
// the signs of (c1, c2, c3) to the column side.  A diagonal tile (a0 == b0) reuses its row-side
// records.
template <bool kSigned>
__device__ __forceinline__ void tan_tile_sum(const float* rec_h, const float4* sgn_h, int a0, int b0,
                                             float (&K)[4][9]) {
    const bool diag = a0 == b0;
    float L[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        L[t] = 0.0f;
#pragma unroll
        for (int k = 0; k < 9; ++k) K[t][k] = 0.0f;
    }
#pragma unroll
    for (int g = 0; g < 8; ++g) {
        const float* pg = rec_h + g * kTanPointStride;
        float ra[2][9], rb[2][9];
        tan_load_record(pg + a0 * kTanRec, ra[0]);
        tan_load_record(pg + (a0 + 1) * kTanRec, ra[1]);
        if (!diag) {
            tan_load_record(pg + b0 * kTanRec, rb[0]);
            tan_load_record(pg + (b0 + 1) * kTanRec, rb[1]);
        } else {
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                rb[0][k] = ra[0][k];
                rb[1][k] = ra[1][k];
            }
        }
        if constexpr (kSigned) {
            const float4 s = sgn_h[g];
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    rb[j][k] *= s.x;
                    rb[j][3 + k] *= s.y;
                    rb[j][6 + k] *= s.z;
                }
        }
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                float* k9 = K[2 * i + j];
                float l = L[2 * i + j];
                l = fmaf(ra[i][0], rb[j][0], l);
                l = fmaf(ra[i][1], rb[j][1], l);
                l = fmaf(ra[i][2], rb[j][2], l);
                L[2 * i + j] = l;
#pragma unroll
                for (int p = 0; p < 3; ++p)
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        k9[3 * p + q] = fmaf(ra[i][3 + p], rb[j][3 + q], k9[3 * p + q]);
                        k9[3 * p + q] = fmaf(ra[i][6 + p], rb[j][6 + q], k9[3 * p + q]);
                    }
            }
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        K[t][0] += L[t];
        K[t][4] += L[t];
        K[t][8] += L[t];
    }
}

__device__ __forceinline__ void bulk_store_s2g(void* dst, const void* src, uint32_t bytes) {
    const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(src));
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(s), "r"(bytes)
                 : "memory");
}

__global__ void __launch_bounds__(kTanThreads, 4) hex_tangent_kernel(int H, const int* __restrict__ idx,
                                                                      const float* __restrict__ invJ,
                                                                      const float* __restrict__ detw,
                                                                      const float* __restrict__ mat,
                                                                      const float4* __restrict__ q4, float lo,
                                                                      float hi, float dt, int64_t trip_off,
                                                                      TripletPlanes vals) {
    extern __shared__ __align__(16) unsigned char smem[];
    float* s_rec = reinterpret_cast<float*>(smem);
    float4* s_x = reinterpret_cast<float4*>(smem + kTanXOff);     // [hex][node]
    float4* s_sgn = reinterpret_cast<float4*>(smem + kTanSgnOff); // [hex][point], padded rows
    float* s_tab = reinterpret_cast<float*>(smem + kTanTabOff);   // [point][node * 3 + axis], padded rows
    const int tid = threadIdx.x;
    const int64_t h0 = (int64_t)blockIdx.x * kTanHex;

    // phase 0: thread (hex, k) stages node k of its hex and loads the data of Gauss point k, so that
    // every global load of the CTA is in flight before the first barrier
    const int64_t he = min(h0 + (tid >> 3), (int64_t)H - 1);  // past the end: a valid hex, never stored
    float ij[9], w = 0.0f, k_mu = 0.0f, k_lambda = 0.0f;
    if (tid < 8 * kTanHex) {
        const int g = tid & 7;
        s_x[tid] = q4[idx[8 * he + g]];
#pragma unroll
        for (int k = 0; k < 9; ++k) ij[k] = invJ[(8 * he + g) * 9 + k];
        w = detw[8 * he + g];
        k_mu = mat[3 * he];
        k_lambda = mat[3 * he + 1];
    }
    for (int i = tid; i < 192; i += kTanThreads) s_tab[(i / 24) * kTanTabStride + i % 24] = (&c_dNdxi[0][0][0])[i];
    __syncthreads();

    // phase 1
    int neg = 0;
    if (tid < 8 * kTanHex) {
        const int hl = tid >> 3, g = tid & 7;
        float d[24];
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const float4 v = reinterpret_cast<const float4*>(s_tab + g * kTanTabStride)[j];
            d[4 * j] = v.x; d[4 * j + 1] = v.y; d[4 * j + 2] = v.z; d[4 * j + 3] = v.w;
        }
        float3 dn[8];
        M3 F;
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const float dx = d[3 * a], dy = d[3 * a + 1], dz = d[3 * a + 2];
            dn[a] = f3(ij[0] * dx + ij[3] * dy + ij[6] * dz, ij[1] * dx + ij[4] * dy + ij[7] * dz,
                       ij[2] * dx + ij[5] * dy + ij[8] * dz);
            const float4 xa = s_x[hl * 8 + a];
            const float xs[3] = {xa.x, xa.y, xa.z};
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                if (a == 0) {
                    F.m[i][0] = xs[i] * dn[a].x;
                    F.m[i][1] = xs[i] * dn[a].y;
                    F.m[i][2] = xs[i] * dn[a].z;
                } else {
                    F.m[i][0] += xs[i] * dn[a].x;
                    F.m[i][1] += xs[i] * dn[a].y;
                    F.m[i][2] += xs[i] * dn[a].z;
                }
            }
        }
        F = clamp_stretch(F, lo, hi);
        const float3 fc0 = col(F, 0), fc1 = col(F, 1), fc2 = col(F, 2);
        const float Ic = dot3(fc0, fc0) + dot3(fc1, fc1) + dot3(fc2, fc2);
        const float Ic1 = fmaxf(Ic + 1.0f, 1.0e-6f);
        const float sdev = 1.0f - 1.0f / Ic1;
        const float coef = k_mu * 2.0f / (Ic1 * Ic1);
        const float c1 = k_mu * sdev * w, c2 = coef * w, c3 = k_lambda * w;
        neg = (c1 < 0.0f) || (c2 < 0.0f) || (c3 < 0.0f);
        s_sgn[hl * kTanSgnStride + g] = make_float4(c1 < 0.0f ? -1.0f : 1.0f, c2 < 0.0f ? -1.0f : 1.0f, c3 < 0.0f ? -1.0f : 1.0f, 0.0f);
        // h sqrt|c| per term, so that products of two records carry h^2 c
        const float q1 = sqrtf(fabsf(c1)) * dt, q2 = sqrtf(fabsf(c2)) * dt, q3 = sqrtf(fabsf(c3)) * dt;
        M3 Fq, Cq;
        const M3 cof = from_cols(cross3(fc1, fc2), cross3(fc2, fc0), cross3(fc0, fc1));
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                Fq.m[i][j] = q2 * F.m[i][j];
                Cq.m[i][j] = q3 * cof.m[i][j];
            }
        float* rp = s_rec + hl * kTanHexStride + g * kTanPointStride;
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const float3 fd = mul(Fq, dn[a]), cd = mul(Cq, dn[a]);
            float4* r4 = reinterpret_cast<float4*>(rp + a * kTanRec);
            r4[0] = make_float4(q1 * dn[a].x, q1 * dn[a].y, q1 * dn[a].z, fd.x);
            r4[1] = make_float4(fd.y, fd.z, cd.x, cd.y);
            rp[a * kTanRec + 8] = cd.z;
        }
    }
    const int any_neg = __syncthreads_or(neg);

    // phase 2
    const int tile = tid / kTanHex, hl = tid - tile * kTanHex;
    int A, B;
    tan_tile_rows(tile, A, B);
    const int a0 = 2 * A, b0 = 2 * B;
    float K[4][9];
    if (any_neg)
        tan_tile_sum<true>(s_rec + hl * kTanHexStride, s_sgn + hl * kTanSgnStride, a0, b0, K);
    else
        tan_tile_sum<false>(s_rec + hl * kTanHexStride, s_sgn + hl * kTanSgnStride, a0, b0, K);
    __syncthreads();  // every record is read before the staging below overwrites them

    // phase 3
    float4* s_A = reinterpret_cast<float4*>(smem + kTanOutA);
    float4* s_B = reinterpret_cast<float4*>(smem + kTanOutB);
    float* s_C = reinterpret_cast<float*>(smem + kTanOutC);
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float* k = K[2 * i + j];
            const int blk = 8 * (a0 + i) + (b0 + j);
            s_A[hl * kTanOut4Stride + blk] = make_float4(k[0], k[1], k[2], k[3]);
            s_B[hl * kTanOut4Stride + blk] = make_float4(k[4], k[5], k[6], k[7]);
            s_C[hl * kTanOut1Stride + blk] = k[8];
            if (A != B) {
                const int tr = 8 * (b0 + j) + (a0 + i);
                s_A[hl * kTanOut4Stride + tr] = make_float4(k[0], k[3], k[6], k[1]);
                s_B[hl * kTanOut4Stride + tr] = make_float4(k[4], k[7], k[2], k[5]);
                s_C[hl * kTanOut1Stride + tr] = k[8];
            }
        }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // staged blocks visible to the bulk copies
    __syncthreads();
    const int nh = (int)min((int64_t)kTanHex, (int64_t)H - h0);
    const int64_t base = trip_off + 64 * h0;
    float* c_dst = vals.c + base;
    const bool c_bulk = (reinterpret_cast<uintptr_t>(c_dst) & 15) == 0;
    const int copies = c_bulk ? 3 * nh : 2 * nh;  // thread k copies plane k % 3 (or % 2) of hex k / 3 (or / 2)
    if (tid < copies) {
        const int per = c_bulk ? 3 : 2, hx = tid / per, plane = tid - hx * per;
        if (plane == 0)
            bulk_store_s2g(vals.a + base + 64 * hx, s_A + hx * kTanOut4Stride, 64 * 16);
        else if (plane == 1)
            bulk_store_s2g(vals.b + base + 64 * hx, s_B + hx * kTanOut4Stride, 64 * 16);
        else
            bulk_store_s2g(c_dst + 64 * hx, s_C + hx * kTanOut1Stride, 64 * 4);
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    }
    if (!c_bulk)
        for (int i = tid; i < nh * 64; i += kTanThreads) c_dst[i] = s_C[(i >> 6) * kTanOut1Stride + (i & 63)];
    if (tid < copies) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // shared memory stays until read
}

}  // namespace

void upload_hex_reference_table() {
    // Once per device.
    static bool done[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
    if (done[dev]) return;
    float table[8][8][3];
    fill_hex_reference_table(table);
    if (cudaMemcpyToSymbol(c_dNdxi, table, sizeof(table)) == cudaSuccess) done[dev] = true;
}

// dN_a/dxi at Gauss point g, evaluated in float32 exactly as the reference's
// _hex_dN_dxi (kernels.py:1356-1419).
void fill_hex_reference_table(float table[8][8][3]) {
    const float gp = 0.5773502691896258f;
    auto sgn_xi = [](int k) { return (k == 1 || k == 2 || k == 5 || k == 6) ? 1.0f : -1.0f; };
    auto sgn_eta = [](int k) { return (k == 2 || k == 3 || k == 6 || k == 7) ? 1.0f : -1.0f; };
    auto sgn_zeta = [](int k) { return (k >= 4) ? 1.0f : -1.0f; };
    for (int g = 0; g < 8; ++g) {
        float xi = sgn_xi(g) * gp, eta = sgn_eta(g) * gp, zeta = sgn_zeta(g) * gp;
        for (int a = 0; a < 8; ++a) {
            float xa = sgn_xi(a), ya = sgn_eta(a), za = sgn_zeta(a);
            table[g][a][0] = xa * (1.0f + ya * eta) * (1.0f + za * zeta) * 0.125f;
            table[g][a][1] = (1.0f + xa * xi) * ya * (1.0f + za * zeta) * 0.125f;
            table[g][a][2] = (1.0f + xa * xi) * (1.0f + ya * eta) * za * 0.125f;
        }
    }
}

cudaError_t launch_node_prepare(Handle& h, float* q, float* v, bool restore_fixed, bool pack_v, bool pack_x,
                                cudaStream_t s) {
    if (h.P == 0) return cudaSuccess;
    node_prepare_kernel<<<blocks_for(h.P, 256), 256, 0, s>>>(h.P, q, v, h.fixed_mask, h.rest, h.dv, h.q4, h.v4, h.x,
                                                             restore_fixed ? 1 : 0, pack_v ? 1 : 0, pack_x ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_element_forces(Handle& h, const float* activations, cudaStream_t s) {
    if (h.T > 0) {
        tet_force_kernel<<<blocks_for(h.T, 128), 128, 0, s>>>(h.T, h.tet_idx, h.tet_pose, h.tet_mat, h.q4, h.v4,
                                                              h.enable_act ? activations : nullptr, h.mu_scale,
                                                              h.min_stretch, h.max_stretch, h.elem_force);
    }
    if (h.H > 0) {
        hex_force_kernel<<<blocks_for(8 * (int64_t)h.H, 256), 256, 0, s>>>(
            h.H, h.hex_idx, h.hex_invJ, h.hex_detw, h.hex_mat, h.q4, h.v4, h.min_stretch, h.max_stretch,
            h.elem_force + 4 * (int64_t)h.T);
    }
    if (h.Tri > 0)
        tri_force_kernel<<<blocks_for(h.Tri, 128), 128, 0, s>>>(h.Tri, h.tri_idx, h.tri_pose, h.tri_mat, h.q4, h.v4,
                                                                h.elem_force + 4 * (int64_t)h.T + 8 * (int64_t)h.H);
    return cudaGetLastError();
}

cudaError_t launch_node_forces(Handle& h, const float* ext, const float* gravity, float dt, int terms, bool scale_by_dt,
                               float* out, cudaStream_t s) {
    if (h.P == 0) return cudaSuccess;
    NodeForceArgs a;
    a.pforce = nullptr;
    a.sc_head = nullptr;
    a.sc_next = nullptr;
    a.sc_force = nullptr;
    a.sforce = nullptr;
    if ((terms & FEM_TERM_SURFACE) && h.sf_active && h.sf_nsurf > 0 && h.sf_nbody > 1) {
        cudaError_t err = launch_surface_contacts(h, s);
        if (err != cudaSuccess) return err;
        a.sforce = h.sf_force;
    }
    if ((terms & FEM_TERM_PARTICLE) && h.pcontact) {
        cudaError_t err = launch_particle_contacts(h, s);
        if (err != cudaSuccess) return err;
        a.pforce = h.pforce;
    }
    if ((terms & FEM_TERM_SOFT_CONTACT) && h.sc_cap > 0) {
        cudaError_t err = launch_soft_contacts(h, s);
        if (err != cudaSuccess) return err;
        a.sc_head = h.sc_head;
        a.sc_next = h.sc_next;
        a.sc_force = h.sc_force;
    }
    a.P = h.P;
    a.T = h.T;
    a.H = h.H;
    a.q4 = h.q4;
    a.v4 = h.v4;
    a.elem_ptr = h.node_elem_ptr;
    a.elem_ent = h.node_elem_ent;
    a.elem_force = h.elem_force;
    a.spring_ptr = h.node_spring_ptr;
    a.spring_ent = h.node_spring_ent;
    a.spring_idx = h.spring_idx;
    a.spring_rest = h.spring_rest;
    a.spring_ke = h.spring_ke;
    a.spring_kd = h.spring_kd;
    a.spring_dir = h.spring_dir;
    a.torque_ke = h.torque_ke;
    a.torque_kd = h.torque_kd;
    a.mass = h.mass;
    a.inv_mass = h.inv_mass;
    a.radius = h.radius;
    a.flags = h.flags;
    a.gravity = gravity != nullptr ? gravity : h.gravity_dev;
    a.ext = ext;
    for (int k = 0; k < 4; ++k) a.ground[k] = h.ground[k];
    a.gke = h.gke;
    a.gkd = h.gkd;
    a.gkf = h.gkf;
    a.gmu = h.gmu;
    a.has_ground = h.has_ground;
    a.linear_damping = h.linear_damping;
    a.dt = dt;
    a.terms = terms;
    a.scale_by_dt = scale_by_dt ? 1 : 0;
    a.out = out;
    const bool full = (h.S > 0 && (terms & FEM_TERM_SPRING)) || a.pforce != nullptr || a.sc_head != nullptr ||
                      a.sforce != nullptr;
    if (full) node_forces_kernel<true><<<blocks_for(h.P, 128), 128, 0, s>>>(a);
    else node_forces_kernel<false><<<blocks_for(h.P, 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_constant_blocks(Handle& h, float dt, cudaStream_t s) {
    if (h.P > 0)
        constant_diag_kernel<<<blocks_for(h.P, 256), 256, 0, s>>>(h.P, h.mass, h.node_spring_ptr, h.node_spring_ent,
                                                                  h.spring_ke, h.spring_kd, dt, h.trip);
    if (h.S > 0)
        constant_offdiag_kernel<<<blocks_for(h.S, 256), 256, 0, s>>>(h.P, h.S, h.spring_ke, h.spring_kd, dt,
                                                                     h.trip);
    if (h.Tri > 0)
        constant_tri_kernel<<<blocks_for(h.Tri, 256), 256, 0, s>>>(h.Tri, h.tri_pose, h.tri_mat, dt,
                                                                   (int64_t)h.P + 2 * (int64_t)h.S, h.trip);
    return cudaGetLastError();
}

cudaError_t launch_element_tangent(Handle& h, float dt, cudaStream_t s) {
    int64_t tet_off = tet_triplet_offset(h);
    if (h.T > 0)
        tet_tangent_kernel<<<blocks_for(h.T, kTetTangentThreads), kTetTangentThreads, 0, s>>>(
            h.T, h.tet_idx, h.tet_pose, h.tet_mat, h.mu_scale, h.q4, h.min_stretch, h.max_stretch, dt, tet_off,
            h.trip);
    if (h.H > 0) {
        cudaError_t err = allow_dynamic_smem((const void*)hex_tangent_kernel, kTanSmemBytes);
        if (err != cudaSuccess) return err;
        hex_tangent_kernel<<<blocks_for(h.H, kTanHex), kTanThreads, kTanSmemBytes, s>>>(
            h.H, h.hex_idx, h.hex_invJ, h.hex_detw, h.hex_mat, h.q4, h.min_stretch, h.max_stretch, dt,
            tet_off + 16 * (int64_t)h.T, h.trip);
    }
    return cudaGetLastError();
}

}  // namespace fem
