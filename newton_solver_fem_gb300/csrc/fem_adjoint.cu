// Adjoint (vector-Jacobian) kernels of one substep with the system matrix held
// fixed -- the reference's differentiation contract (differentiation.py:1-8,
// 287-394): A dv = h f(q, v, a) - h^2 K v, dv = A^-1 rhs, v' = v + dv,
// q' = q + h v'.  Given the gradient of the total force g = dL/df, these
// kernels give dL/dq, dL/dv (and dL/d activation, dL/d shear scale) of
//   tet force      kernels.py:511-632 (+ activation 484-508)
//   hex force      kernels.py:1481-1601
//   springs        kernels.py:176-218 (+ bend torque 221-291)
//   triangles      kernels.py:876-960
//   ground         kernels.py:1132-1195
//   damping        kernels.py:1289-1307
// and of the elastic predictor rhs -= sum_j A_ij (v_j - v_i) plus the spring
// damping term (implicit_predictor.py:9-41).  The linear solve's VJP is a
// second solve with the same symmetric A (fem_solve).  The stretch clamp is
// differentiated as the identity: exact while every principal stretch lies
// inside [min_stretch, max_stretch] (the clamp leaves F unchanged), which is the
// regime of the differentiable workloads.
// Element gradients go to per-element slots and are summed per node in a
// fixed order, like the forward forces: no float atomics.
#include <string>

#include "fem_generic.cuh"
#include "fem_internal.cuh"
#include "fem_math.cuh"

namespace fem {
namespace {
__constant__ float c_dNdxi[8][8][3];  // this translation unit's copy of the Gauss table
}  // namespace

void upload_hex_reference_table_adjoint() {
    static bool done[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
    if (done[dev]) return;
    float table[8][8][3];
    fill_hex_reference_table(table);
    if (cudaMemcpyToSymbol(c_dNdxi, table, sizeof(table)) == cudaSuccess) done[dev] = true;
}

namespace {

__device__ __forceinline__ float3 ld3(const float* p, int i) { return f3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ void add3(float* p, int i, float3 v) {
    p[3 * i] += v.x;
    p[3 * i + 1] += v.y;
    p[3 * i + 2] += v.z;
}

// F-bar contribution of J = det F: dJ/dF = cof(F) (columns c1 x c2, c2 x c0, c0 x c1).
__device__ __forceinline__ M3 cofactor(const M3& F) {
    float3 c0 = col(F, 0), c1 = col(F, 1), c2 = col(F, 2);
    return from_cols(cross3(c1, c2), cross3(c2, c0), cross3(c0, c1));
}

// Per-element outputs: written (acc == 0) or accumulated over calls (acc != 0).
__device__ __forceinline__ void put(float* p, size_t i, float v, int acc) {
    if (acc) p[i] += v;
    else p[i] = v;
}

// Tet4 force VJP.  g (scaled by gs) is the gradient of the loss wrt every node's
// restoring force; writes the per-corner position / velocity gradients and,
// when given, dL/d activation, dL/d shear scale and dL/d (mu, lambda, k_d) of
// the raw material row (the shear scale multiplies mu; alpha depends on both).
__global__ void tet_force_vjp_kernel(int T, const int4* __restrict__ idx, const float* __restrict__ pose,
                                     const float* __restrict__ mat, const float* __restrict__ mu_scale,
                                     const float4* __restrict__ q4, const float4* __restrict__ v4,
                                     const float* __restrict__ act, const float* __restrict__ g, float gs, float lo,
                                     float hi, float4* __restrict__ grad, float* __restrict__ act_bar,
                                     float* __restrict__ scale_bar, float* __restrict__ mat_bar, int acc) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    float4* o = grad + 8 * (size_t)t;  // [corner][x-bar, v-bar]
    float mu0 = mat[3 * t], lam = mat[3 * t + 1], kd = mat[3 * t + 2];
    float sc = mu_scale != nullptr ? mu_scale[t] : 1.0f;
    float mu = mu0 * sc;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (mu == 0.0f && lam == 0.0f && kd == 0.0f) {  // skipped element (kernels.py:545-548): no dependence
        for (int k = 0; k < 8; ++k) o[k] = zero4;
        if (act_bar) put(act_bar, t, 0.0f, acc);
        if (scale_bar) put(scale_bar, t, 0.0f, acc);
        if (mat_bar)
            for (int k = 0; k < 3; ++k) put(mat_bar, 3 * (size_t)t + k, 0.0f, acc);
        return;
    }
    int4 n = idx[t];
    float3 x0 = xyz(q4[n.x]), x1 = xyz(q4[n.y]), x2 = xyz(q4[n.z]), x3 = xyz(q4[n.w]);
    float3 v0 = xyz(v4[n.x]), v1 = xyz(v4[n.y]), v2 = xyz(v4[n.z]), v3 = xyz(v4[n.w]);
    float3 g0 = ld3(g, n.x) * gs, g1 = ld3(g, n.y) * gs, g2 = ld3(g, n.z) * gs, g3 = ld3(g, n.w) * gs;
    float3 e[3] = {x1 - x0, x2 - x0, x3 - x0};
    float3 ve[3] = {v1 - v0, v2 - v0, v3 - v0};
    M3 Dm;
#pragma unroll
    for (int k = 0; k < 9; ++k) Dm.m[k / 3][k % 3] = pose[9 * t + k];
    float irv = det3(Dm) * 6.0f;
    float rv = 1.0f / irv;
    float alpha = 1.0f + mu / lam - mu / (4.0f * lam);
    float kmu = mu * rv, klam = lam * rv, kdm = kd * rv;
    M3 F = clamp_stretch(matmul(from_cols(e[0], e[1], e[2]), Dm), lo, hi);
    float Ic = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Ic += F.m[i][j] * F.m[i][j];
    float c = kmu * (1.0f - 1.0f / (Ic + 1.0f));
    float J = det3(F);
    float Jc = fmaxf(J, 0.01f);
    float s = irv / 6.0f;
    float3 d[3] = {cross3(e[1], e[2]) * s, cross3(e[2], e[0]) * s, cross3(e[0], e[1]) * s};
    const float dsum = dot3(d[0], ve[0]) + dot3(d[1], ve[1]) + dot3(d[2], ve[2]);  // dJ/dt
    float ft = (Jc - alpha) * klam + dsum * kdm;
    // gradient wrt f_a (a = 1..3): restoring r_a = -f_a and r_0 = f_1 + f_2 + f_3
    float3 G[3] = {g0 - g1, g0 - g2, g0 - g3};
    float3 eb[3] = {f3(0.f, 0.f, 0.f), f3(0.f, 0.f, 0.f), f3(0.f, 0.f, 0.f)};
    float3 veb[3] = {f3(0.f, 0.f, 0.f), f3(0.f, 0.f, 0.f), f3(0.f, 0.f, 0.f)};
    float lam_act_b = 0.0f;  // dL/d lambda through the activation term
    if (act != nullptr) {  // r_1 -= fb etc.: the activation terms enter like f_1..f_3
        float scA = lam * act[t] / 6.0f;
        float3 cr[3] = {cross3(e[1], e[2]), cross3(e[2], e[0]), cross3(e[0], e[1])};
        const float s_act = dot3(G[0], cr[0]) + dot3(G[1], cr[1]) + dot3(G[2], cr[2]);
        if (act_bar) put(act_bar, t, s_act * lam / 6.0f, acc);
        lam_act_b = s_act * act[t] / 6.0f;
        float3 cb0 = G[0] * scA, cb1 = G[1] * scA, cb2 = G[2] * scA;
        eb[1] = eb[1] + cross3(e[2], cb0);
        eb[2] = eb[2] + cross3(cb0, e[1]);
        eb[2] = eb[2] + cross3(e[0], cb1);
        eb[0] = eb[0] + cross3(cb1, e[2]);
        eb[0] = eb[0] + cross3(e[1], cb2);
        eb[1] = eb[1] + cross3(cb2, e[0]);
    } else if (act_bar) {
        put(act_bar, t, 0.0f, acc);
    }
    // f_a = (P Dm^T)[:, a-1] + d_a ft
    M3 Pb;  // P-bar = H-bar Dm, H-bar columns = G_a
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float gi[3] = {i == 0 ? G[0].x : (i == 1 ? G[0].y : G[0].z), i == 0 ? G[1].x : (i == 1 ? G[1].y : G[1].z),
                       i == 0 ? G[2].x : (i == 1 ? G[2].y : G[2].z)};
#pragma unroll
        for (int j = 0; j < 3; ++j) Pb.m[i][j] = gi[0] * Dm.m[0][j] + gi[1] * Dm.m[1][j] + gi[2] * Dm.m[2][j];
    }
    float3 db[3] = {G[0] * ft, G[1] * ft, G[2] * ft};
    float ftb = dot3(G[0], d[0]) + dot3(G[1], d[1]) + dot3(G[2], d[2]);
    float Jcb = ftb * klam;
    float alphab = -ftb * klam;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        db[a] = db[a] + ve[a] * (ftb * kdm);
        veb[a] = veb[a] + d[a] * (ftb * kdm);
    }
    // P = c F + kdm dF
    const M3 dF = matmul(from_cols(ve[0], ve[1], ve[2]), Dm);
    float cb = 0.0f, dfb = 0.0f;  // dL/dc and the P-bar : dF part of dL/dkdm
    M3 Fb, dFb;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            Fb.m[i][j] = c * Pb.m[i][j];
            dFb.m[i][j] = kdm * Pb.m[i][j];
            cb += Pb.m[i][j] * F.m[i][j];
            dfb += Pb.m[i][j] * dF.m[i][j];
        }
    float Icb = cb * kmu / ((Ic + 1.0f) * (Ic + 1.0f));
    float kmub = cb * (1.0f - 1.0f / (Ic + 1.0f));
    M3 cof = cofactor(F);
    float Jb = J > 0.01f ? Jcb : 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Fb.m[i][j] += 2.0f * Icb * F.m[i][j] + Jb * cof.m[i][j];
    // d_a = s (e_b x e_c)
    eb[1] = eb[1] + cross3(e[2], db[0]) * s;
    eb[2] = eb[2] + cross3(db[0], e[1]) * s;
    eb[2] = eb[2] + cross3(e[0], db[1]) * s;
    eb[0] = eb[0] + cross3(db[1], e[2]) * s;
    eb[0] = eb[0] + cross3(e[1], db[2]) * s;
    eb[1] = eb[1] + cross3(db[2], e[0]) * s;
    // F = Ds Dm, dF = Dv Dm: edge a-bar = (F-bar Dm^T)[:, a]
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float3 dm = row(Dm, a);
        eb[a] = eb[a] + mul(Fb, dm);
        veb[a] = veb[a] + mul(dFb, dm);
    }
    float3 x0b = -(eb[0] + eb[1] + eb[2]), v0b = -(veb[0] + veb[1] + veb[2]);
    o[0] = f4(x0b);
    o[1] = f4(v0b);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        o[2 + 2 * a] = f4(eb[a]);
        o[3 + 2 * a] = f4(veb[a]);
    }
    if (scale_bar) put(scale_bar, t, kmub * mu0 * rv + alphab * 0.75f * mu0 / lam, acc);
    if (mat_bar) {
        // kmu = mu0 sc / V, klam = lam / V, kdm = kd / V, alpha = 1 + 0.75 mu0 sc / lam
        const float klamb = ftb * (Jc - alpha);
        const float kdmb = dfb + ftb * dsum;
        put(mat_bar, 3 * (size_t)t, kmub * sc * rv + alphab * 0.75f * sc / lam, acc);
        put(mat_bar, 3 * (size_t)t + 1, klamb * rv - alphab * 0.75f * mu / (lam * lam) + lam_act_b, acc);
        put(mat_bar, 3 * (size_t)t + 2, kdmb * rv, acc);
    }
}

// Lane g of an 8-lane group handles Gauss point g of one hex.  g is scaled by
// gs; mat_bar (optional) receives dL/d (mu, lambda, k_d) of the element.
__global__ void hex_force_vjp_kernel(int H, const int* __restrict__ idx, const float* __restrict__ invJ,
                                     const float* __restrict__ detw, const float* __restrict__ mat,
                                     const float4* __restrict__ q4, const float4* __restrict__ v4,
                                     const float* __restrict__ g, float gs, float lo, float hi,
                                     float4* __restrict__ grad, float* __restrict__ mat_bar, int acc) {
    int gid = blockIdx.x * blockDim.x + threadIdx.x;
    int h = gid >> 3, gp = gid & 7;
    bool live = h < H;
    int he = live ? h : H - 1;
    int node = idx[8 * he + gp];
    float3 xg = xyz(q4[node]), vg = xyz(v4[node]), gg = ld3(g, node) * gs;
    float mu = mat[3 * he], lam = mat[3 * he + 1], kd = mat[3 * he + 2];
    float alpha = 1.0f + mu / lam - mu / (4.0f * lam);
    M3 iJ;
#pragma unroll
    for (int k = 0; k < 9; ++k) iJ.m[k / 3][k % 3] = invJ[(8 * he + gp) * 9 + k];
    float w = detw[8 * he + gp];
    int base = threadIdx.x & 24;
    float3 dN[8], gb[8];
    M3 F, dF;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) F.m[i][j] = dF.m[i][j] = 0.0f;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        float3 xa = f3(__shfl_sync(0xffffffffu, xg.x, base + a), __shfl_sync(0xffffffffu, xg.y, base + a),
                       __shfl_sync(0xffffffffu, xg.z, base + a));
        float3 va = f3(__shfl_sync(0xffffffffu, vg.x, base + a), __shfl_sync(0xffffffffu, vg.y, base + a),
                       __shfl_sync(0xffffffffu, vg.z, base + a));
        gb[a] = f3(__shfl_sync(0xffffffffu, gg.x, base + a), __shfl_sync(0xffffffffu, gg.y, base + a),
                   __shfl_sync(0xffffffffu, gg.z, base + a));
        dN[a] = mulT(iJ, f3(c_dNdxi[gp][a][0], c_dNdxi[gp][a][1], c_dNdxi[gp][a][2]));
        float xs[3] = {xa.x, xa.y, xa.z}, vs[3] = {va.x, va.y, va.z};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            F.m[i][0] += xs[i] * dN[a].x;
            F.m[i][1] += xs[i] * dN[a].y;
            F.m[i][2] += xs[i] * dN[a].z;
            dF.m[i][0] += vs[i] * dN[a].x;
            dF.m[i][1] += vs[i] * dN[a].y;
            dF.m[i][2] += vs[i] * dN[a].z;
        }
    }
    F = clamp_stretch(F, lo, hi);
    float Ic = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Ic += F.m[i][j] * F.m[i][j];
    float c = mu * (1.0f - 1.0f / (Ic + 1.0f));
    float J = det3(F);
    float Jc = fmaxf(J, 0.01f);
    M3 cof = cofactor(F);
    float vol = lam * (Jc - alpha);
    // restoring r_a = -sum_g w P dN_a  =>  P-bar = -w sum_a g_a (outer) dN_a
    M3 Pb;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Pb.m[i][j] = 0.0f;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        float gs[3] = {gb[a].x, gb[a].y, gb[a].z}, ds[3] = {dN[a].x, dN[a].y, dN[a].z};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Pb.m[i][j] -= w * gs[i] * ds[j];
    }
    float cb = 0.0f, volb = 0.0f;
    M3 Fb, dFb, cofb;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            Fb.m[i][j] = c * Pb.m[i][j];
            dFb.m[i][j] = kd * Pb.m[i][j];
            cofb.m[i][j] = vol * Pb.m[i][j];
            cb += Pb.m[i][j] * F.m[i][j];
            volb += Pb.m[i][j] * cof.m[i][j];
        }
    float Icb = cb * mu / ((Ic + 1.0f) * (Ic + 1.0f));
    float Jb = J > 0.01f ? volb * lam : 0.0f;
    if (mat_bar != nullptr) {  // c = mu (1 - 1/(Ic+1)), vol = lam (Jc - alpha), alpha = 1 + 0.75 mu / lam
        float mb = cb * (1.0f - 1.0f / (Ic + 1.0f)) - 0.75f * volb;
        float lb = volb * (Jc - alpha) + 0.75f * volb * mu / lam;
        float kb = 0.0f;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) kb += Pb.m[i][j] * dF.m[i][j];
#pragma unroll
        for (int off = 1; off < 8; off <<= 1) {  // sum over the element's 8 Gauss points, fixed order
            mb += __shfl_xor_sync(0xffffffffu, mb, off);
            lb += __shfl_xor_sync(0xffffffffu, lb, off);
            kb += __shfl_xor_sync(0xffffffffu, kb, off);
        }
        if (live && gp == 0) {
            put(mat_bar, 3 * (size_t)h, mb, acc);
            put(mat_bar, 3 * (size_t)h + 1, lb, acc);
            put(mat_bar, 3 * (size_t)h + 2, kb, acc);
        }
    }
    float3 c0 = col(F, 0), c1 = col(F, 1), c2 = col(F, 2);
    float3 k0 = col(cofb, 0), k1 = col(cofb, 1), k2 = col(cofb, 2);
    float3 c0b = cross3(k1, c2) + cross3(c1, k2);  // from col1 = c2 x c0 and col2 = c0 x c1
    float3 c1b = cross3(c2, k0) + cross3(k2, c0);  // from col0 = c1 x c2 and col2
    float3 c2b = cross3(k0, c1) + cross3(c0, k1);  // from col0 and col1
    M3 cb3 = from_cols(c0b, c1b, c2b);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Fb.m[i][j] += 2.0f * Icb * F.m[i][j] + Jb * cof.m[i][j] + cb3.m[i][j];
    float3 xm = f3(0.f, 0.f, 0.f), vm = f3(0.f, 0.f, 0.f);
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        float3 xa = mul(Fb, dN[a]), va = mul(dFb, dN[a]);
#pragma unroll
        for (int off = 1; off < 8; off <<= 1) {
            xa.x += __shfl_xor_sync(0xffffffffu, xa.x, off);
            xa.y += __shfl_xor_sync(0xffffffffu, xa.y, off);
            xa.z += __shfl_xor_sync(0xffffffffu, xa.z, off);
            va.x += __shfl_xor_sync(0xffffffffu, va.x, off);
            va.y += __shfl_xor_sync(0xffffffffu, va.y, off);
            va.z += __shfl_xor_sync(0xffffffffu, va.z, off);
        }
        if (a == gp) {
            xm = xa;
            vm = va;
        }
    }
    if (live) {
        grad[2 * (8 * (size_t)h + gp)] = f4(xm);
        grad[2 * (8 * (size_t)h + gp) + 1] = f4(vm);
    }
}

__device__ __forceinline__ void seed(V3<Dual>& a, int k) {
    if (k == 0) a.x.d = 1.0f;
    else if (k == 1) a.y.d = 1.0f;
    else a.z.d = 1.0f;
}

// Triangle VJP by forward-mode differentiation of the shared force: one dual
// pass per input component (x0..x2, v0..v2) gives a Jacobian column, dotted
// with the corners' force gradients.  Slots [corner][x-bar, v-bar].
__global__ void tri_force_vjp_kernel(int Tri, const int* __restrict__ idx, const float4* __restrict__ pose,
                                     const float* __restrict__ mat, const float4* __restrict__ q4,
                                     const float4* __restrict__ v4, const float* __restrict__ g, float gs,
                                     float4* __restrict__ grad) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= Tri) return;
    int n[3];
    float3 xs[3], vs[3], gc[3];
    float m[5];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        n[c] = idx[3 * e + c];
        xs[c] = xyz(q4[n[c]]);
        vs[c] = xyz(v4[n[c]]);
        gc[c] = ld3(g, n[c]) * gs;
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) m[k] = mat[5 * e + k];
    const float4 Dm = pose[e];
    float bar[18];  // [x0 x1 x2 v0 v1 v2] components
    for (int dir = 0; dir < 18; ++dir) {
        V3<Dual> x[3], v[3], f[3];
        for (int c = 0; c < 3; ++c) {
            x[c] = lift3<Dual>(xs[c]);
            v[c] = lift3<Dual>(vs[c]);
        }
        seed(dir < 9 ? x[dir / 3] : v[(dir - 9) / 3], dir % 3);
        triangle_force(x, v, Dm, m, f);
        float acc = 0.0f;
        for (int c = 0; c < 3; ++c) acc += gc[c].x * f[c].x.d + gc[c].y * f[c].y.d + gc[c].z * f[c].z.d;
        bar[dir] = acc;
    }
    for (int c = 0; c < 3; ++c) {
        grad[2 * (3 * (size_t)e + c)] = make_float4(bar[3 * c], bar[3 * c + 1], bar[3 * c + 2], 0.0f);
        grad[2 * (3 * (size_t)e + c) + 1] = make_float4(bar[9 + 3 * c], bar[9 + 3 * c + 1], bar[9 + 3 * c + 2], 0.0f);
    }
}

// VJP of one spring's bend torque wrt xij and vij (the torque enters node j
// with + and node i with -): dual passes over the six inputs.
__device__ void spring_torque_vjp(float3 xij, float3 vij, float3 dir0, float kt, float kwt, float3 tbar,
                                  float3& xijb, float3& vijb) {
    float bar[6];
    for (int k = 0; k < 6; ++k) {
        V3<Dual> x = lift3<Dual>(xij), v = lift3<Dual>(vij), out;
        seed(k < 3 ? x : v, k % 3);
        bar[k] = spring_torque_force(x, v, dir0, kt, kwt, out)
                     ? tbar.x * out.x.d + tbar.y * out.y.d + tbar.z * out.z.d
                     : 0.0f;
    }
    xijb = f3(bar[0], bar[1], bar[2]);
    vijb = f3(bar[3], bar[4], bar[5]);
}

struct NodeVjpArgs {
    int P, T;
    const float4* q4;
    const float4* v4;
    const float* g;
    const int* elem_ptr;
    const int* elem_ent;
    const float4* elem_grad;
    const int* spring_ptr;
    const int* spring_ent;
    const int* spring_idx;
    const float* spring_rest;
    const float* spring_ke;
    const float* spring_kd;
    const float* spring_dir;
    float torque_ke, torque_kd;
    const float* mass;
    const float* inv_mass;
    const float* radius;
    const int* flags;
    const float* gravity;
    float ground[4];
    float gke, gkd, gkf, gmu;
    int has_ground;
    float linear_damping;
    float gs;                           // scale of g
    const unsigned char* fixed_mask;    // non-null: zero q_bar and v_bar at fixed nodes at the end
    float* ext_bar;                     // non-null: ext_bar += gs g (a load enters the force as h ext)
    float* q_bar;
    float* v_bar;
};

__global__ void node_vjp_kernel(NodeVjpArgs a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.P) return;
    float3 xb = f3(0.f, 0.f, 0.f), vb = f3(0.f, 0.f, 0.f);
    for (int e = a.elem_ptr[i]; e < a.elem_ptr[i + 1]; ++e) {
        int ent = a.elem_ent[e];
        xb = xb + xyz(a.elem_grad[2 * (size_t)ent]);
        vb = vb + xyz(a.elem_grad[2 * (size_t)ent + 1]);
    }
    for (int e = a.spring_ptr[i]; e < a.spring_ptr[i + 1]; ++e) {
        int ent = a.spring_ent[e];
        int s = ent >> 1;
        int ia = a.spring_idx[2 * s], ib = a.spring_idx[2 * s + 1];
        if (ia < 0 || ib < 0) continue;
        float3 xij = xyz(a.q4[ia]) - xyz(a.q4[ib]);
        float3 vij = xyz(a.v4[ia]) - xyz(a.v4[ib]);
        float L = len3(xij);
        if (L < 1.0e-6f) continue;
        float3 dir = f3(xij.x / L, xij.y / L, xij.z / L);
        float cc = L - a.spring_rest[s];
        float dcdt = dot3(dir, vij);
        float m = a.spring_ke[s] * cc + a.spring_kd[s] * dcdt;
        float3 fsb = (ld3(a.g, ib) - ld3(a.g, ia)) * a.gs;  // f_a = -fs, f_b = +fs
        float3 dirb = fsb * m;
        float mb = dot3(fsb, dir);
        float Lb = mb * a.spring_ke[s];
        float dcdtb = mb * a.spring_kd[s];
        dirb = dirb + vij * dcdtb;
        float3 vijb = dir * dcdtb;
        float3 xijb = (dirb - dir * dot3(dir, dirb)) * (1.0f / L) + dir * Lb;
        if (a.spring_dir != nullptr) {
            const float3 d0 = f3(a.spring_dir[3 * s], a.spring_dir[3 * s + 1], a.spring_dir[3 * s + 2]);
            float3 txb, tvb;
            spring_torque_vjp(xij, vij, d0, a.torque_ke, a.torque_kd, fsb, txb, tvb);
            xijb = xijb + txb;
            vijb = vijb + tvb;
        }
        if (ent & 1) {
            xb = xb - xijb;
            vb = vb - vijb;
        } else {
            xb = xb + xijb;
            vb = vb + vijb;
        }
    }
    bool active = (a.flags[i] & 1) != 0;
    float3 gi = ld3(a.g, i) * a.gs;
    if (a.ext_bar != nullptr) add3(a.ext_bar, i, gi);
    if (a.has_ground && active) {
        float3 n = f3(a.ground[0], a.ground[1], a.ground[2]);
        float3 xi = xyz(a.q4[i]), vi = xyz(a.v4[i]);
        float c = fminf(dot3(n, xi) + a.ground[3] - a.radius[i], 0.0f);
        if (c < 0.0f) {
            float vn = dot3(n, vi);
            float fn = c * a.gke + fminf(vn, 0.0f) * a.gkd;
            float3 vt_raw = vi - n * vn;
            float vs = len3(vt_raw);
            float3 vt = vs > 0.0f ? vt_raw * (1.0f / vs) : vt_raw;
            float3 grav = f3(a.gravity[0], a.gravity[1], a.gravity[2]);
            float inv_m = a.inv_mass[i];
            float m = inv_m > 0.0f ? 1.0f / fmaxf(inv_m, 1e-9f) : 0.0f;
            float cap = m * len3(grav);
            float fn_eff = fminf(fabsf(fn), cap);
            float ft = fminf(vs * a.gkf, a.gmu * fn_eff);
            // f = -n fn - vt ft
            float fnb = -dot3(n, gi);
            float3 vtb = gi * (-ft);
            float ftb = -dot3(vt, gi);
            float vsb = 0.0f;
            if (vs * a.gkf < a.gmu * fn_eff) vsb += ftb * a.gkf;
            else if (fabsf(fn) < cap) fnb += ftb * a.gmu * (fn >= 0.0f ? 1.0f : -1.0f);
            float3 vt_rawb = f3(0.f, 0.f, 0.f);
            if (vs > 0.0f) vt_rawb = (vtb - vt * dot3(vt, vtb)) * (1.0f / vs) + vt * vsb;
            float vnb = vn < 0.0f ? fnb * a.gkd : 0.0f;
            xb = xb + n * (fnb * a.gke);
            vb = vb + vt_rawb - n * dot3(n, vt_rawb) + n * vnb;
        }
    }
    if (active && a.linear_damping > 0.0f) vb = vb + gi * (-a.linear_damping * a.mass[i]);
    if (a.fixed_mask != nullptr && a.fixed_mask[i]) {  // fixed inputs are overwritten by the restore
        for (int c = 0; c < 3; ++c) a.q_bar[3 * i + c] = a.v_bar[3 * i + c] = 0.0f;
        return;
    }
    add3(a.q_bar, i, xb);
    add3(a.v_bar, i, vb);
}

// Seed of one substep's adjoint: the outputs' gradients (zero at fixed nodes,
// which the restore overwrites) give vt = v'-bar + h q'-bar, the right-hand
// side of the adjoint solve; v-bar restarts from vt (v' = v + dv) and q-bar
// keeps q'-bar (q' = q + h v').
__global__ void adjoint_seed_kernel(int P, float h, const unsigned char* __restrict__ fixed, float* __restrict__ q_bar,
                                    float* __restrict__ v_bar, float* __restrict__ vt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const bool fx = fixed[i] != 0;
    float3 qb = fx ? f3(0.f, 0.f, 0.f) : ld3(q_bar, i);
    float3 vb = fx ? f3(0.f, 0.f, 0.f) : ld3(v_bar, i);
    float3 w = vb + qb * h;
    for (int c = 0; c < 3; ++c) {
        const float wc = c == 0 ? w.x : (c == 1 ? w.y : w.z);
        const float qc = c == 0 ? qb.x : (c == 1 ? qb.y : qb.z);
        vt[3 * i + c] = wc;
        v_bar[3 * i + c] = wc;
        q_bar[3 * i + c] = qc;
    }
}

__global__ void pack_adjoint_start_kernel(int P, const float* __restrict__ x, const unsigned char* __restrict__ fixed,
                                          float4* __restrict__ x4) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    x4[i] = fixed[i] ? make_float4(0.f, 0.f, 0.f, 0.f) : f4(ld3(x, i));
}

// v-bar += -(A rbar)_k + (sum_j A_kj)^T rbar_k  and the spring damping term.
__global__ void predictor_vjp_kernel(int nslices, const int* __restrict__ slice_ptr, const int2* __restrict__ meta,
                                     const unsigned* __restrict__ row_info, const float4* __restrict__ valA,
                                     const float4* __restrict__ valB, const float* __restrict__ valC,
                                     const int* __restrict__ scol, const float* __restrict__ rb,
                                     const int* __restrict__ sptr, const int* __restrict__ sent,
                                     const int* __restrict__ sidx, const float* __restrict__ skd, float dt,
                                     float* __restrict__ v_bar) {
    int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (warp_global >= nslices) return;
    int2 m = meta[warp_global];
    if (lane >= m.y) return;
    int row = m.x + lane;
    int len = (int)(row_info[row] & ~kFixedBit);
    int base = slice_ptr[warp_global];
    float3 ar = f3(0.f, 0.f, 0.f);
    float R[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int k = 0; k < len; ++k) {
        size_t e = (size_t)(base + k) * kSlice + lane;
        float4 A = valA[e], B = valB[e];
        float C = valC[e];
        float3 p = ld3(rb, scol[e]);
        ar = ar + f3(A.x * p.x + A.y * p.y + A.z * p.z, A.w * p.x + B.x * p.y + B.y * p.z,
                     B.z * p.x + B.w * p.y + C * p.z);
        R[0] += A.x; R[1] += A.y; R[2] += A.z; R[3] += A.w; R[4] += B.x;
        R[5] += B.y; R[6] += B.z; R[7] += B.w; R[8] += C;
    }
    float3 r = ld3(rb, row);
    float3 rt = f3(R[0] * r.x + R[3] * r.y + R[6] * r.z, R[1] * r.x + R[4] * r.y + R[7] * r.z,
                   R[2] * r.x + R[5] * r.y + R[8] * r.z);
    float3 vb = rt - ar;
    for (int e = sptr[row]; e < sptr[row + 1]; ++e) {
        int ent = sent[e];
        int s = ent >> 1;
        int ia = sidx[2 * s], ib = sidx[2 * s + 1];
        if (ia < 0 || ib < 0) continue;
        float3 d = (ld3(rb, ia) - ld3(rb, ib)) * (dt * skd[s]);
        vb = (ent & 1) ? vb - d : vb + d;
    }
    add3(v_bar, row, vb);
}

}  // namespace
}  // namespace fem

using fem::Handle;

namespace {
int adj_cuda(cudaError_t e) { return fem::report_cuda(e); }
struct AdjDeviceGuard {
    int prev = -1;
    explicit AdjDeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~AdjDeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};
}  // namespace

namespace {

int adjoint_supported(const Handle& h, const char* who) {
    if (h.pcontact || h.sc_cap > 0 || h.sf_active)
        return fem::report(FEM_ERR_UNSUPPORTED,
                           (std::string(who) + ": particle, soft and surface contacts are not differentiated "
                                               "(fixed-matrix contract)").c_str());
    return FEM_OK;
}

template <class T>
int lazy_alloc(Handle& h, T*& ptr, size_t count) {
    if (ptr != nullptr || count == 0) return FEM_OK;
    void* p = nullptr;
    if (cudaError_t e = cudaMalloc(&p, count * sizeof(T)); e != cudaSuccess) return fem::report_cuda(e);
    h.allocations.push_back(p);
    ptr = static_cast<T*>(p);
    return FEM_OK;
}

// Adjoint scratch, allocated by the first VJP or adjoint call (call once before capturing).
int ensure_adjoint_scratch(Handle& h) {
    const size_t slots = 2 * (4 * (size_t)h.T + 8 * (size_t)h.H + 3 * (size_t)h.Tri);
    int code = lazy_alloc(h, h.elem_grad, slots);
    if (code == FEM_OK) code = lazy_alloc(h, h.adj_vt, 3 * (size_t)h.P);
    if (code == FEM_OK) code = lazy_alloc(h, h.adj_x, 3 * (size_t)h.P);
    if (code == FEM_OK) code = lazy_alloc(h, h.roll_f, 3 * (size_t)h.P);
    return code;
}

// Element and node VJPs of the force terms at the packed state (h.q4, h.v4) for
// the force gradient gs * g.  Per-element outputs are written, or accumulated
// when `accumulate`; ext_bar (optional) accumulates gs * g; with zero_fixed the
// node gradients end zero at fixed nodes.
cudaError_t launch_force_vjp(Handle& h, const float* activations, const float* gravity, const float* g, float gs,
                             float* q_bar, float* v_bar, float* act_bar, float* scale_bar, float* tet_mat_bar,
                             float* hex_mat_bar, float* ext_bar, bool accumulate, bool zero_fixed, cudaStream_t s) {
    const int acc = accumulate ? 1 : 0;
    if (h.T > 0)
        fem::tet_force_vjp_kernel<<<(h.T + 127) / 128, 128, 0, s>>>(
            h.T, h.tet_idx, h.tet_pose, h.tet_mat, h.mu_scale, h.q4, h.v4, h.enable_act ? activations : nullptr, g,
            gs, h.min_stretch, h.max_stretch, h.elem_grad, act_bar, scale_bar, tet_mat_bar, acc);
    if (h.H > 0)
        fem::hex_force_vjp_kernel<<<(int)((8 * (int64_t)h.H + 255) / 256), 256, 0, s>>>(
            h.H, h.hex_idx, h.hex_invJ, h.hex_detw, h.hex_mat, h.q4, h.v4, g, gs, h.min_stretch, h.max_stretch,
            h.elem_grad + 2 * 4 * (size_t)h.T, hex_mat_bar, acc);
    if (h.Tri > 0)
        fem::tri_force_vjp_kernel<<<(h.Tri + 127) / 128, 128, 0, s>>>(
            h.Tri, h.tri_idx, h.tri_pose, h.tri_mat, h.q4, h.v4, g, gs,
            h.elem_grad + 2 * (4 * (size_t)h.T + 8 * (size_t)h.H));
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    fem::NodeVjpArgs a;
    a.P = h.P;
    a.T = h.T;
    a.q4 = h.q4;
    a.v4 = h.v4;
    a.g = g;
    a.gs = gs;
    a.elem_ptr = h.node_elem_ptr;
    a.elem_ent = h.node_elem_ent;
    a.elem_grad = h.elem_grad;
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
    for (int k = 0; k < 4; ++k) a.ground[k] = h.ground[k];
    a.gke = h.gke;
    a.gkd = h.gkd;
    a.gkf = h.gkf;
    a.gmu = h.gmu;
    a.has_ground = h.has_ground;
    a.linear_damping = h.linear_damping;
    a.fixed_mask = zero_fixed ? h.fixed_mask : nullptr;
    a.ext_bar = ext_bar;
    a.q_bar = q_bar;
    a.v_bar = v_bar;
    fem::node_vjp_kernel<<<(h.P + 127) / 128, 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_predictor_vjp(Handle& h, const float* rhs_bar, float dt, float* v_bar, cudaStream_t s) {
    const int threads = 256;
    const int blocks = (h.nslices * 32 + threads - 1) / threads;
    fem::predictor_vjp_kernel<<<blocks, threads, 0, s>>>(h.nslices, h.slice_ptr, h.slice_meta, h.row_info, h.valA,
                                                          h.valB, h.valC, h.scol, rhs_bar, h.node_spring_ptr,
                                                          h.node_spring_ent, h.spring_idx, h.spring_kd, dt, v_bar);
    return cudaGetLastError();
}

// One substep of the differentiable forward (SolverFEM.step on the fixed matrix): the state
// (q_in, v_in) -> (q_out, v_out) through the handle's step kernels.  Without warm start the
// solve starts from zero, like the reference's checked solves.
cudaError_t rollout_substep(Handle& h, float* q_in, float* v_in, float* q_out, float* v_out, const float* ext,
                            const float* act, const float* gravity, float dt, float tol, int maxiter, bool warm,
                            cudaStream_t s) {
    cudaError_t err = cudaSuccess;
    if (!warm) err = cudaMemsetAsync(h.dv, 0, sizeof(float) * 3 * (size_t)h.P, s);
    if (err == cudaSuccess) err = fem::launch_node_prepare(h, q_in, v_in, true, true, true, s);
    if (err == cudaSuccess) err = fem::launch_element_forces(h, act, s);
    if (err == cudaSuccess) err = fem::launch_node_forces(h, ext, gravity, dt, FEM_TERM_ALL, true, h.roll_f, s);
    if (err == cudaSuccess) err = fem::launch_pcg(h, dt, 1, q_out, v_out, h.roll_f, s, nullptr, nullptr, tol, maxiter);
    return err;
}

// fem_refresh_tangent without the dt change: the tangent at q (fixed nodes restored in place).
cudaError_t refresh_at(Handle& h, float* q, cudaStream_t s) {
    cudaError_t err = fem::launch_node_prepare(h, q, nullptr, true, false, false, s);
    if (err == cudaSuccess) err = fem::launch_element_tangent(h, h.dt, s);
    if (err == cudaSuccess) err = fem::launch_gather(h, s);
    return err;
}

int rollout_args_ok(const Handle& h, int substeps, float dt, float tol, int maxiter, const char* who) {
    const char* why = nullptr;
    if (substeps < 0) why = ": substeps must be non-negative";
    else if (!(dt > 0.0f) || dt != h.dt) why = ": dt must equal the assembled timestep (the matrix is held fixed)";
    else if (!(tol > 0.0f) || maxiter < 0) why = ": tolerance must be positive and maxiter non-negative";
    if (why == nullptr) return FEM_OK;
    return fem::report(FEM_ERR_BAD_ARG, (std::string(who) + why).c_str());
}

}  // namespace

extern "C" {

int fem_set_mu_scale(FemHandle* H, const float* scale) {
    if (H == nullptr) return fem::report(FEM_ERR_BAD_ARG, "fem_set_mu_scale: null handle");
    H->h.mu_scale = scale;
    return FEM_OK;
}

int fem_solve(FemHandle* H, const float* rhs, float* x, float tolerance, int32_t maxiter, void* stream) {
    if (H == nullptr || rhs == nullptr || x == nullptr) return fem::report(FEM_ERR_BAD_ARG, "fem_solve: null argument");
    if (!(tolerance > 0.0f) || maxiter < 0)
        return fem::report(FEM_ERR_BAD_ARG, "fem_solve: tolerance must be positive and maxiter non-negative");
    Handle& h = H->h;
    if (h.P == 0) return FEM_OK;
    AdjDeviceGuard g(H->device);
    return adj_cuda(fem::launch_pcg(h, h.dt, 0, nullptr, nullptr, nullptr, (cudaStream_t)stream, rhs, x, tolerance,
                                    maxiter));
}

int fem_force_vjp(FemHandle* H, const float* q, const float* v, const float* activations, const float* gravity,
                  const float* force_bar, float* q_bar, float* v_bar, float* activation_bar, float* mu_scale_bar,
                  void* stream) {
    return fem_force_vjp_materials(H, q, v, activations, gravity, force_bar, q_bar, v_bar, activation_bar,
                                   mu_scale_bar, nullptr, nullptr, stream);
}

int fem_force_vjp_materials(FemHandle* H, const float* q, const float* v, const float* activations,
                            const float* gravity, const float* force_bar, float* q_bar, float* v_bar,
                            float* activation_bar, float* mu_scale_bar, float* tet_material_bar,
                            float* hex_material_bar, void* stream) {
    if (H == nullptr || q == nullptr || v == nullptr || force_bar == nullptr || q_bar == nullptr || v_bar == nullptr)
        return fem::report(FEM_ERR_BAD_ARG, "fem_force_vjp: null argument");
    Handle& h = H->h;
    if (h.P == 0) return FEM_OK;
    if (int code = adjoint_supported(h, "fem_force_vjp"); code != FEM_OK) return code;
    AdjDeviceGuard g(H->device);
    cudaStream_t s = (cudaStream_t)stream;
    if (int code = ensure_adjoint_scratch(h); code != FEM_OK) return code;
    cudaError_t err = fem::launch_node_prepare(h, const_cast<float*>(q), const_cast<float*>(v), false, true, false, s);
    if (err == cudaSuccess)
        err = launch_force_vjp(h, activations, gravity, force_bar, 1.0f, q_bar, v_bar, activation_bar, mu_scale_bar,
                               tet_material_bar, hex_material_bar, nullptr, false, false, s);
    return adj_cuda(err);
}

int fem_predictor_vjp(FemHandle* H, const float* rhs_bar, float dt, float* v_bar, void* stream) {
    if (H == nullptr || rhs_bar == nullptr || v_bar == nullptr)
        return fem::report(FEM_ERR_BAD_ARG, "fem_predictor_vjp: null argument");
    Handle& h = H->h;
    if (h.P == 0) return FEM_OK;
    AdjDeviceGuard g(H->device);
    return adj_cuda(launch_predictor_vjp(h, rhs_bar, dt, v_bar, (cudaStream_t)stream));
}

int fem_rollout_segment(FemHandle* H, const float* q0, const float* v0, const float* dv0, int32_t substeps,
                        const float* external_forces, const float* activations, const float* gravity, float dt,
                        float tolerance, int32_t maxiter, int32_t warm_start, int32_t refresh, float* q_states,
                        float* v_states, float* dv_out, void* stream) {
    if (H == nullptr || q0 == nullptr || v0 == nullptr || q_states == nullptr || v_states == nullptr)
        return fem::report(FEM_ERR_BAD_ARG, "fem_rollout_segment: null argument");
    Handle& h = H->h;
    if (int code = rollout_args_ok(h, substeps, dt, tolerance, maxiter, "fem_rollout_segment"); code != FEM_OK)
        return code;
    if (h.enable_act && h.T > 0 && activations == nullptr)
        return fem::report(FEM_ERR_BAD_ARG, "fem_rollout_segment: tet activations are enabled but none were passed");
    if (h.P == 0) return FEM_OK;
    if (int code = adjoint_supported(h, "fem_rollout_segment"); code != FEM_OK) return code;
    AdjDeviceGuard g(H->device);
    if (int code = ensure_adjoint_scratch(h); code != FEM_OK) return code;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n3 = 3 * (size_t)h.P;
    cudaError_t err = cudaSuccess;
    if (q0 != q_states) err = cudaMemcpyAsync(q_states, q0, n3 * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess && v0 != v_states)
        err = cudaMemcpyAsync(v_states, v0, n3 * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess && refresh) err = refresh_at(h, q_states, s);
    if (err == cudaSuccess && warm_start) {
        if (dv0 != nullptr) err = cudaMemcpyAsync(h.dv, dv0, n3 * sizeof(float), cudaMemcpyDeviceToDevice, s);
        else err = cudaMemsetAsync(h.dv, 0, n3 * sizeof(float), s);
    }
    for (int k = 0; k < substeps && err == cudaSuccess; ++k)
        err = rollout_substep(h, q_states + k * n3, v_states + k * n3, q_states + (k + 1) * n3,
                              v_states + (k + 1) * n3, external_forces, activations, gravity, dt, tolerance, maxiter,
                              warm_start != 0, s);
    if (err == cudaSuccess && dv_out != nullptr)
        err = cudaMemcpyAsync(dv_out, h.dv, n3 * sizeof(float), cudaMemcpyDeviceToDevice, s);
    return adj_cuda(err);
}

int fem_adjoint_segment(FemHandle* H, float* q_states, float* v_states, int32_t substeps,
                        const float* external_forces, const float* activations, const float* gravity, float dt,
                        float tolerance, int32_t maxiter, int32_t refresh, float* adjoint_start, float* q_bar,
                        float* v_bar, float* ext_bar, float* activation_bar, float* mu_scale_bar,
                        float* tet_material_bar, float* hex_material_bar, void* stream) {
    if (H == nullptr || q_states == nullptr || v_states == nullptr || q_bar == nullptr || v_bar == nullptr)
        return fem::report(FEM_ERR_BAD_ARG, "fem_adjoint_segment: null argument");
    Handle& h = H->h;
    if (int code = rollout_args_ok(h, substeps, dt, tolerance, maxiter, "fem_adjoint_segment"); code != FEM_OK)
        return code;
    if (h.enable_act && h.T > 0 && activations == nullptr)
        return fem::report(FEM_ERR_BAD_ARG, "fem_adjoint_segment: tet activations are enabled but none were passed");
    if (h.P == 0) return FEM_OK;
    if (int code = adjoint_supported(h, "fem_adjoint_segment"); code != FEM_OK) return code;
    AdjDeviceGuard g(H->device);
    if (int code = ensure_adjoint_scratch(h); code != FEM_OK) return code;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n3 = 3 * (size_t)h.P;
    const int threads = 256, blocks = (h.P + threads - 1) / threads;
    (void)external_forces;  // the force VJP does not depend on the load (it enters the force linearly)
    cudaError_t err = refresh ? refresh_at(h, q_states, s) : cudaSuccess;
    float* rb = adjoint_start != nullptr ? adjoint_start : h.adj_x;  // the adjoint solution (and warm start)
    for (int k = substeps - 1; k >= 0 && err == cudaSuccess; --k) {
        fem::adjoint_seed_kernel<<<blocks, threads, 0, s>>>(h.P, dt, h.fixed_mask, q_bar, v_bar, h.adj_vt);
        err = cudaGetLastError();
        if (err == cudaSuccess && adjoint_start != nullptr) {
            fem::pack_adjoint_start_kernel<<<blocks, threads, 0, s>>>(h.P, rb, h.fixed_mask, h.x);
            err = cudaGetLastError();
        }
        if (err == cudaSuccess)
            err = fem::launch_pcg(h, dt, 0, nullptr, nullptr, nullptr, s, h.adj_vt, rb, tolerance, maxiter,
                                  adjoint_start != nullptr);
        if (err == cudaSuccess) err = launch_predictor_vjp(h, rb, dt, v_bar, s);
        if (err == cudaSuccess)
            err = fem::launch_node_prepare(h, q_states + k * n3, v_states + k * n3, false, true, false, s);
        if (err == cudaSuccess)
            err = launch_force_vjp(h, activations, gravity, rb, dt, q_bar, v_bar, activation_bar, mu_scale_bar,
                                   tet_material_bar, hex_material_bar, ext_bar, true, true, s);
    }
    return adj_cuda(err);
}

}  // extern "C"
