/*
 * fem_port.c -- TEST INFRASTRUCTURE ONLY: a float32 C/OpenMP restatement of the
 * SolverFEM per-substep hot path, used as the CPU baseline (bench.py's
 * cpu_baseline leg and --impl reference) and checked against the NumPy oracle
 * in tests.  It never runs on the product path.
 *
 * Reference algorithm followed (src/newton_solver_fem/_src/solvers/fem/):
 *   tet force          kernels.py:511-632     tet tangent   kernels.py:635-850
 *   hex force          kernels.py:1481-1601   hex tangent   kernels.py:1609-1747
 *   springs            kernels.py:176-218, 294-366   spring damping restore  implicit_predictor.py:26-41
 *   ground, gravity    kernels.py:1132-1195, 1273-1307
 *   block inverse      kernels.py:1817-1849   predictor     implicit_predictor.py:9-41
 *   RHS normalisation  kernels.py:1779-1814   solve         solver.py:1254-1351 (Warp cg semantics)
 * Element forces go to per-element buffers and are gathered per node in a fixed
 * order (the reference uses float atomics); the principal-stretch clamp uses the
 * same sufficient in-range test as the GPU kernels and otherwise a Jacobi
 * eigen-decomposition of F^T F (Golub & Van Loan sec. 8.5).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { float m[3][3]; } M3;

static float det3(const M3* a) {
    return a->m[0][0] * (a->m[1][1] * a->m[2][2] - a->m[1][2] * a->m[2][1]) -
           a->m[0][1] * (a->m[1][0] * a->m[2][2] - a->m[1][2] * a->m[2][0]) +
           a->m[0][2] * (a->m[1][0] * a->m[2][1] - a->m[1][1] * a->m[2][0]);
}

static void cross3(const float* a, const float* b, float* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

static float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static void jacobi_rotate(float c[3][3], float v[3][3], int p, int q) {
    float apq = c[p][q];
    if (fabsf(apq) < 1e-30f) return;
    float tau = (c[q][q] - c[p][p]) / (2.0f * apq);
    float t = copysignf(1.0f, tau) / (fabsf(tau) + sqrtf(1.0f + tau * tau));
    float cs = 1.0f / sqrtf(1.0f + t * t), sn = t * cs;
    for (int k = 0; k < 3; ++k) {
        float a = c[k][p], b = c[k][q];
        c[k][p] = cs * a - sn * b;
        c[k][q] = sn * a + cs * b;
    }
    for (int k = 0; k < 3; ++k) {
        float a = c[p][k], b = c[q][k];
        c[p][k] = cs * a - sn * b;
        c[q][k] = sn * a + cs * b;
    }
    for (int k = 0; k < 3; ++k) {
        float a = v[k][p], b = v[k][q];
        v[k][p] = cs * a - sn * b;
        v[k][q] = sn * a + cs * b;
    }
}

/* principal-stretch clamp with signed smallest stretch (rotation-variant SVD) */
static void clamp_stretch(M3* F, float lo, float hi) {
    if (lo < 0.0f || hi < 0.0f) return;
    float ic = 0.0f;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) ic += F->m[i][j] * F->m[i][j];
    float J = det3(F);
    if (J > 0.0f && ic <= hi * hi && 2.0f * J >= lo * ic) return;
    float c[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            c[i][j] = F->m[0][i] * F->m[0][j] + F->m[1][i] * F->m[1][j] + F->m[2][i] * F->m[2][j];
    for (int s = 0; s < 6; ++s) {
        jacobi_rotate(c, v, 0, 1);
        jacobi_rotate(c, v, 0, 2);
        jacobi_rotate(c, v, 1, 2);
    }
    float ev[3] = {c[0][0], c[1][1], c[2][2]};
    int o[3] = {0, 1, 2};
    for (int a = 0; a < 3; ++a)
        for (int b = a + 1; b < 3; ++b)
            if (ev[o[a]] < ev[o[b]]) { int t = o[a]; o[a] = o[b]; o[b] = t; }
    float V[3][3], U[3][3], s[3];
    for (int k = 0; k < 3; ++k) { V[k][0] = v[k][o[0]]; V[k][1] = v[k][o[1]]; }
    float v0[3] = {V[0][0], V[1][0], V[2][0]}, v1[3] = {V[0][1], V[1][1], V[2][1]}, v2[3];
    cross3(v0, v1, v2);
    float b[3][3];
    float* vv[3] = {v0, v1, v2};
    for (int k = 0; k < 3; ++k)
        for (int i = 0; i < 3; ++i) b[k][i] = F->m[i][0] * vv[k][0] + F->m[i][1] * vv[k][1] + F->m[i][2] * vv[k][2];
    float u0[3], u1[3], u2[3];
    s[0] = sqrtf(dot3(b[0], b[0]));
    if (s[0] > 1e-30f) for (int i = 0; i < 3; ++i) u0[i] = b[0][i] / s[0];
    else { u0[0] = 1; u0[1] = 0; u0[2] = 0; }
    float d = dot3(u0, b[1]);
    for (int i = 0; i < 3; ++i) u1[i] = b[1][i] - u0[i] * d;
    s[1] = sqrtf(dot3(u1, u1));
    if (s[1] > 1e-30f) for (int i = 0; i < 3; ++i) u1[i] /= s[1];
    else {
        float t[3] = {fabsf(u0[0]) < 0.9f ? 1.f : 0.f, fabsf(u0[0]) < 0.9f ? 0.f : 1.f, 0.f};
        cross3(u0, t, u1);
        float n = sqrtf(dot3(u1, u1));
        for (int i = 0; i < 3; ++i) u1[i] /= n;
    }
    cross3(u0, u1, u2);
    s[2] = dot3(u2, b[2]);
    for (int k = 0; k < 3; ++k) s[k] = fmaxf(fminf(s[k], hi), lo);
    for (int i = 0; i < 3; ++i) { U[i][0] = u0[i]; U[i][1] = u1[i]; U[i][2] = u2[i]; }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            F->m[i][j] = U[i][0] * s[0] * vv[0][j] + U[i][1] * s[1] * vv[1][j] + U[i][2] * s[2] * vv[2][j];
}

static void hex_dNdxi(float out[8][8][3]) {
    const float gp = 0.5773502691896258f;
    for (int g = 0; g < 8; ++g) {
        float xi = ((g == 1 || g == 2 || g == 5 || g == 6) ? 1.f : -1.f) * gp;
        float eta = ((g == 2 || g == 3 || g == 6 || g == 7) ? 1.f : -1.f) * gp;
        float zeta = (g >= 4 ? 1.f : -1.f) * gp;
        for (int a = 0; a < 8; ++a) {
            float xa = (a == 1 || a == 2 || a == 5 || a == 6) ? 1.f : -1.f;
            float ya = (a == 2 || a == 3 || a == 6 || a == 7) ? 1.f : -1.f;
            float za = a >= 4 ? 1.f : -1.f;
            out[g][a][0] = xa * (1.0f + ya * eta) * (1.0f + za * zeta) * 0.125f;
            out[g][a][1] = (1.0f + xa * xi) * ya * (1.0f + za * zeta) * 0.125f;
            out[g][a][2] = (1.0f + xa * xi) * (1.0f + ya * eta) * za * 0.125f;
        }
    }
}

int port_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Per-element restoring forces of Tet4 elements into out[4T][3]. */
void port_tet_forces(int64_t T, const int32_t* idx, const float* pose, const float* mat, const float* q,
                     const float* v, float lo, float hi, float* out) {
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < T; ++t) {
        float* o = out + 12 * t;
        float mu = mat[3 * t], lam = mat[3 * t + 1], kd = mat[3 * t + 2];
        if (mu == 0.f && lam == 0.f && kd == 0.f) { memset(o, 0, 12 * sizeof(float)); continue; }
        const int32_t* n = idx + 4 * t;
        float x[4][3], vv[4][3];
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 3; ++c) { x[a][c] = q[3 * n[a] + c]; vv[a][c] = v[3 * n[a] + c]; }
        float e[3][3], ev[3][3];
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) { e[a][c] = x[a + 1][c] - x[0][c]; ev[a][c] = vv[a + 1][c] - vv[0][c]; }
        M3 Dm;
        for (int k = 0; k < 9; ++k) Dm.m[k / 3][k % 3] = pose[9 * t + k];
        float irv = det3(&Dm) * 6.0f, rv = 1.0f / irv;
        float alpha = 1.0f + mu / lam - mu / (4.0f * lam);
        float kmu = mu * rv, klam = lam * rv, kdamp = kd * rv;
        M3 F, dF;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                F.m[i][j] = e[0][i] * Dm.m[0][j] + e[1][i] * Dm.m[1][j] + e[2][i] * Dm.m[2][j];
                dF.m[i][j] = ev[0][i] * Dm.m[0][j] + ev[1][i] * Dm.m[1][j] + ev[2][i] * Dm.m[2][j];
            }
        clamp_stretch(&F, lo, hi);
        float Ic = 0.f;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Ic += F.m[i][j] * F.m[i][j];
        float sdev = kmu * (1.0f - 1.0f / (Ic + 1.0f));
        M3 P;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) P.m[i][j] = F.m[i][j] * sdev + dF.m[i][j] * kdamp;
        float f[4][3];
        for (int a = 0; a < 3; ++a)
            for (int i = 0; i < 3; ++i)
                f[a + 1][i] = P.m[i][0] * Dm.m[a][0] + P.m[i][1] * Dm.m[a][1] + P.m[i][2] * Dm.m[a][2];
        float J = fmaxf(det3(&F), 0.01f), s = irv / 6.0f;
        float d[3][3];
        cross3(e[1], e[2], d[0]);
        cross3(e[2], e[0], d[1]);
        cross3(e[0], e[1], d[2]);
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) d[a][c] *= s;
        float ft = (J - alpha) * klam + (dot3(d[0], ev[0]) + dot3(d[1], ev[1]) + dot3(d[2], ev[2])) * kdamp;
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) f[a + 1][c] += d[a][c] * ft;
        for (int c = 0; c < 3; ++c) f[0][c] = -(f[1][c] + f[2][c] + f[3][c]);
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 3; ++c) o[3 * a + c] = -f[a][c];
    }
}

/* Per-element restoring forces of Hex8 elements into out[8H][3]. */
void port_hex_forces(int64_t H, const int32_t* idx, const float* invJ, const float* detw, const float* mat,
                     const float* q, const float* v, float lo, float hi, float* out) {
    float dxi[8][8][3];
    hex_dNdxi(dxi);
#pragma omp parallel for schedule(static)
    for (int64_t h = 0; h < H; ++h) {
        float mu = mat[3 * h], lam = mat[3 * h + 1], kd = mat[3 * h + 2];
        float alpha = 1.0f + mu / lam - mu / (4.0f * lam);
        float x[8][3], vv[8][3], acc[8][3];
        memset(acc, 0, sizeof(acc));
        for (int a = 0; a < 8; ++a)
            for (int c = 0; c < 3; ++c) { x[a][c] = q[3 * idx[8 * h + a] + c]; vv[a][c] = v[3 * idx[8 * h + a] + c]; }
        for (int g = 0; g < 8; ++g) {
            const float* iJ = invJ + (8 * h + g) * 9;
            float dN[8][3];
            for (int a = 0; a < 8; ++a)
                for (int c = 0; c < 3; ++c)
                    dN[a][c] = iJ[c] * dxi[g][a][0] + iJ[3 + c] * dxi[g][a][1] + iJ[6 + c] * dxi[g][a][2];
            M3 F, dF;
            memset(&F, 0, sizeof(F));
            memset(&dF, 0, sizeof(dF));
            for (int a = 0; a < 8; ++a)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) { F.m[i][j] += x[a][i] * dN[a][j]; dF.m[i][j] += vv[a][i] * dN[a][j]; }
            clamp_stretch(&F, lo, hi);
            float c0[3] = {F.m[0][0], F.m[1][0], F.m[2][0]}, c1[3] = {F.m[0][1], F.m[1][1], F.m[2][1]},
                  c2[3] = {F.m[0][2], F.m[1][2], F.m[2][2]};
            float Ic = dot3(c0, c0) + dot3(c1, c1) + dot3(c2, c2);
            float sdev = mu * (1.0f - 1.0f / (Ic + 1.0f));
            float J = fmaxf(det3(&F), 0.01f), vol = lam * (J - alpha);
            float k0[3], k1[3], k2[3];
            cross3(c1, c2, k0);
            cross3(c2, c0, k1);
            cross3(c0, c1, k2);
            M3 P;
            for (int i = 0; i < 3; ++i) {
                float cof[3] = {k0[i], k1[i], k2[i]};
                for (int j = 0; j < 3; ++j) P.m[i][j] = (F.m[i][j] * sdev + dF.m[i][j] * kd) + cof[j] * vol;
            }
            float w = detw[8 * h + g];
            for (int a = 0; a < 8; ++a)
                for (int i = 0; i < 3; ++i)
                    acc[a][i] += (P.m[i][0] * dN[a][0] + P.m[i][1] * dN[a][1] + P.m[i][2] * dN[a][2]) * w;
        }
        for (int a = 0; a < 8; ++a)
            for (int c = 0; c < 3; ++c) out[24 * h + 3 * a + c] = -acc[a][c];
    }
}

/* Tet4 tangent blocks into vals[16T][9] (h^2 scaled). */
void port_tet_tangent(int64_t T, const int32_t* idx, const float* pose, const float* mat, const float* q, float lo,
                      float hi, float dt, float* vals) {
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < T; ++t) {
        float* o = vals + 144 * t;
        float mu = mat[3 * t], lam = mat[3 * t + 1];
        M3 Dm;
        for (int k = 0; k < 9; ++k) Dm.m[k / 3][k % 3] = pose[9 * t + k];
        float irv = det3(&Dm) * 6.0f;
        if ((mu == 0.f && lam == 0.f && mat[3 * t + 2] == 0.f) || irv <= 0.0f) { memset(o, 0, 144 * sizeof(float)); continue; }
        const int32_t* n = idx + 4 * t;
        float e[3][3];
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) e[a][c] = q[3 * n[a + 1] + c] - q[3 * n[0] + c];
        float rv = 1.0f / irv, kmu = mu * rv, klam = lam * rv;
        M3 F;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) F.m[i][j] = e[0][i] * Dm.m[0][j] + e[1][i] * Dm.m[1][j] + e[2][i] * Dm.m[2][j];
        clamp_stretch(&F, lo, hi);
        float Ic = 0.f;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Ic += F.m[i][j] * F.m[i][j];
        float Ic1 = fmaxf(Ic + 1.0f, 1e-6f), s = 1.0f - 1.0f / Ic1, coef = kmu * 2.0f / (Ic1 * Ic1);
        float sv = irv / 6.0f, dJ[4][3], dm[4][3], Fd[4][3];
        cross3(e[1], e[2], dJ[1]);
        cross3(e[2], e[0], dJ[2]);
        cross3(e[0], e[1], dJ[3]);
        for (int c = 0; c < 3; ++c) {
            for (int a = 1; a < 4; ++a) { dJ[a][c] *= sv; dm[a][c] = Dm.m[a - 1][c]; }
            dJ[0][c] = -(dJ[1][c] + dJ[2][c] + dJ[3][c]);
            dm[0][c] = -(dm[1][c] + dm[2][c] + dm[3][c]);
        }
        for (int a = 0; a < 4; ++a)
            for (int i = 0; i < 3; ++i) Fd[a][i] = F.m[i][0] * dm[a][0] + F.m[i][1] * dm[a][1] + F.m[i][2] * dm[a][2];
        float scale = dt * dt;
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) {
                float diag = kmu * s * dot3(dm[a], dm[b]);
                float* blk = o + 9 * (4 * a + b);
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j)
                        blk[3 * i + j] = ((i == j ? diag : 0.f) + Fd[a][i] * Fd[b][j] * coef + dJ[a][i] * dJ[b][j] * klam) * scale;
            }
    }
}

/* Hex8 tangent blocks into vals[64H][9] (h^2 scaled). */
void port_hex_tangent(int64_t H, const int32_t* idx, const float* invJ, const float* detw, const float* mat,
                      const float* q, float lo, float hi, float dt, float* vals) {
    float dxi[8][8][3];
    hex_dNdxi(dxi);
#pragma omp parallel for schedule(static)
    for (int64_t h = 0; h < H; ++h) {
        float mu = mat[3 * h], lam = mat[3 * h + 1];
        float x[8][3];
        for (int a = 0; a < 8; ++a)
            for (int c = 0; c < 3; ++c) x[a][c] = q[3 * idx[8 * h + a] + c];
        float K[64][9];
        memset(K, 0, sizeof(K));
        for (int g = 0; g < 8; ++g) {
            const float* iJ = invJ + (8 * h + g) * 9;
            float dN[8][3], Fd[8][3], cd[8][3];
            for (int a = 0; a < 8; ++a)
                for (int c = 0; c < 3; ++c)
                    dN[a][c] = iJ[c] * dxi[g][a][0] + iJ[3 + c] * dxi[g][a][1] + iJ[6 + c] * dxi[g][a][2];
            M3 F;
            memset(&F, 0, sizeof(F));
            for (int a = 0; a < 8; ++a)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) F.m[i][j] += x[a][i] * dN[a][j];
            clamp_stretch(&F, lo, hi);
            float c0[3] = {F.m[0][0], F.m[1][0], F.m[2][0]}, c1[3] = {F.m[0][1], F.m[1][1], F.m[2][1]},
                  c2[3] = {F.m[0][2], F.m[1][2], F.m[2][2]};
            float Ic1 = fmaxf(dot3(c0, c0) + dot3(c1, c1) + dot3(c2, c2) + 1.0f, 1e-6f);
            float s = 1.0f - 1.0f / Ic1, coef = mu * 2.0f / (Ic1 * Ic1), w = detw[8 * h + g];
            float k0[3], k1[3], k2[3];
            cross3(c1, c2, k0);
            cross3(c2, c0, k1);
            cross3(c0, c1, k2);
            for (int a = 0; a < 8; ++a)
                for (int i = 0; i < 3; ++i) {
                    Fd[a][i] = F.m[i][0] * dN[a][0] + F.m[i][1] * dN[a][1] + F.m[i][2] * dN[a][2];
                    cd[a][i] = k0[i] * dN[a][0] + k1[i] * dN[a][1] + k2[i] * dN[a][2];
                }
            for (int a = 0; a < 8; ++a)
                for (int b = 0; b < 8; ++b) {
                    float diag = mu * s * dot3(dN[a], dN[b]);
                    float* kb = K[8 * a + b];
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j)
                            kb[3 * i + j] += ((i == j ? diag : 0.f) + Fd[a][i] * Fd[b][j] * coef + cd[a][i] * cd[b][j] * lam) * w;
                }
        }
        float scale = dt * dt;
        for (int k = 0; k < 64 * 9; ++k) vals[576 * h + k] = ((float*)K)[k] * scale;
    }
}

/* Linear spring + damping forces (kernels.py:176-218) into out[2S][3]: entry 2s
 * is the force on the first endpoint, 2s+1 on the second (zero for springs with
 * a negative index or a length below 1e-6). */
void port_spring_forces(int64_t S, const int32_t* idx, const float* rest, const float* ke, const float* kd,
                        const float* q, const float* v, float* out) {
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < S; ++s) {
        float* o = out + 6 * s;
        memset(o, 0, 6 * sizeof(float));
        int32_t i = idx[2 * s], j = idx[2 * s + 1];
        if (i < 0 || j < 0) continue;
        float xij[3], vij[3];
        for (int c = 0; c < 3; ++c) {
            xij[c] = q[3 * (int64_t)i + c] - q[3 * (int64_t)j + c];
            vij[c] = v[3 * (int64_t)i + c] - v[3 * (int64_t)j + c];
        }
        float L = sqrtf(dot3(xij, xij));
        if (L < 1.0e-6f) continue;
        float d[3] = {xij[0] / L, xij[1] / L, xij[2] / L};
        float m = ke[s] * (L - rest[s]) + kd[s] * dot3(d, vij);
        for (int c = 0; c < 3; ++c) {
            o[c] = -d[c] * m;
            o[3 + c] = d[c] * m;
        }
    }
}

/* values[slot] = sum of trip[contrib[c]] for c in [cptr[slot], cptr[slot+1]) in order. */
void port_gather(int64_t nnzb, const int32_t* cptr, const int32_t* contrib, const float* trip, float* values) {
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < nnzb; ++j) {
        float b[9] = {0};
        for (int c = cptr[j]; c < cptr[j + 1]; ++c)
            for (int k = 0; k < 9; ++k) b[k] += trip[9 * (int64_t)contrib[c] + k];
        memcpy(values + 9 * j, b, sizeof(b));
    }
}

/* out[i] = sum over entries e in [ptr[i], ptr[i+1]) of buf[ent[e]] (3-vectors). */
void port_node_gather(int64_t n, const int32_t* ptr, const int32_t* ent, const float* buf, float* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float s[3] = {0, 0, 0};
        for (int e = ptr[i]; e < ptr[i + 1]; ++e)
            for (int c = 0; c < 3; ++c) s[c] += buf[3 * (int64_t)ent[e] + c];
        for (int c = 0; c < 3; ++c) out[3 * i + c] = s[c];
    }
}

static void block_inverse(const float* blk, float* out) {
    float scale = fmaxf(fabsf(blk[0]), fmaxf(fabsf(blk[4]), fabsf(blk[8])));
    if (scale > 0.0f) {
        float a[9];
        for (int k = 0; k < 9; ++k) a[k] = blk[k] / scale;
        float tr = (a[0] + a[4] + a[8]) / 3.0f;
        float c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8], c02 = a[3] * a[7] - a[4] * a[6];
        float det = a[0] * c00 + a[1] * c01 + a[2] * c02;
        if (tr > 0.0f && fabsf(det) > 1.0e-9f * tr * tr * tr) {
            float id = 1.0f / det;
            float r[9] = {c00, a[2] * a[7] - a[1] * a[8], a[1] * a[5] - a[2] * a[4],
                          c01, a[0] * a[8] - a[2] * a[6], a[2] * a[3] - a[0] * a[5],
                          c02, a[1] * a[6] - a[0] * a[7], a[0] * a[4] - a[1] * a[3]};
            for (int k = 0; k < 9; ++k) out[k] = r[k] * id / scale;
            return;
        }
    }
    memset(out, 0, 9 * sizeof(float));
    out[0] = blk[0] > 0.f ? 1.0f / blk[0] : 1.0f;
    out[4] = blk[4] > 0.f ? 1.0f / blk[4] : 1.0f;
    out[8] = blk[8] > 0.f ? 1.0f / blk[8] : 1.0f;
}

void port_block_jacobi(int64_t n, const int32_t* off, const int32_t* col, const float* val, float* minv) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float d[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        for (int k = off[i]; k < off[i + 1]; ++k)
            if (col[k] == i) memcpy(d, val + 9 * (int64_t)k, sizeof(d));
        block_inverse(d, minv + 9 * i);
    }
}

static void spmv(int64_t n, const int32_t* off, const int32_t* col, const float* val, const unsigned char* fixed,
                 const float* x, float* y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float s[3] = {0, 0, 0};
        if (fixed[i]) {
            for (int c = 0; c < 3; ++c) y[3 * i + c] = x[3 * i + c];
            continue;
        }
        for (int k = off[i]; k < off[i + 1]; ++k) {
            const float* a = val + 9 * (int64_t)k;
            const float* p = x + 3 * (int64_t)col[k];
            if (fixed[col[k]]) continue;
            s[0] += a[0] * p[0] + a[1] * p[1] + a[2] * p[2];
            s[1] += a[3] * p[0] + a[4] * p[1] + a[5] * p[2];
            s[2] += a[6] * p[0] + a[7] * p[1] + a[8] * p[2];
        }
        for (int c = 0; c < 3; ++c) y[3 * i + c] = s[c];
    }
}

static double dotv(int64_t m, const float* a, const float* b) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t k = 0; k < m; ++k) s += (double)a[k] * b[k];
    return s;
}

static void precond(int64_t n, const float* minv, const float* r, float* z) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const float* m = minv + 9 * i;
        const float* v = r + 3 * i;
        for (int c = 0; c < 3; ++c) z[3 * i + c] = m[3 * c] * v[0] + m[3 * c + 1] * v[1] + m[3 * c + 2] * v[2];
    }
}

/*
 * One substep's linear solve and integration for a single scene.  f holds
 * h*sum(f) on entry and the final RHS on exit; dv holds the warm start and
 * receives the increment; work needs 5*3*n floats.  Returns the iteration count.
 */
int port_solve(int64_t n, const int32_t* off, const int32_t* col, const float* val, const float* minv,
               const unsigned char* fixed, const float* rest, const float* q, const float* v, float* f, float* dv,
               float* q_out, float* v_out, float dt, float tol, int maxiter, float* work) {
    float *x = work, *r = work + 3 * n, *z = work + 6 * n, *p = work + 9 * n, *y = work + 12 * n;
    float mx = 0.0f;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float rhs[3] = {0, 0, 0};
        if (!fixed[i]) {
            float cv[3] = {0, 0, 0};
            for (int k = off[i]; k < off[i + 1]; ++k) {
                const float* a = val + 9 * (int64_t)k;
                int j = col[k];
                float d[3] = {v[3 * j] - v[3 * i], v[3 * j + 1] - v[3 * i + 1], v[3 * j + 2] - v[3 * i + 2]};
                cv[0] += a[0] * d[0] + a[1] * d[1] + a[2] * d[2];
                cv[1] += a[3] * d[0] + a[4] * d[1] + a[5] * d[2];
                cv[2] += a[6] * d[0] + a[7] * d[1] + a[8] * d[2];
            }
            for (int c = 0; c < 3; ++c) rhs[c] = f[3 * i + c] - cv[c];
        }
        for (int c = 0; c < 3; ++c) {
            f[3 * i + c] = rhs[c];
            mx = fmaxf(mx, fabsf(rhs[c]));
            x[3 * i + c] = fixed[i] ? 0.0f : dv[3 * i + c];
        }
    }
    float scale = (mx > 0.0f && mx < 1.0e-12f) ? fminf(1.0f / mx, 1.0e30f) : 1.0f;
    int64_t m = 3 * n;
    for (int64_t k = 0; k < m; ++k) x[k] = (mx == 0.0f) ? 0.0f : scale * x[k];
    spmv(n, off, col, val, fixed, x, y);
    for (int64_t k = 0; k < m; ++k) r[k] = scale * f[k] - y[k];
    double rr = dotv(m, r, r), bb = 0.0;
    for (int64_t k = 0; k < m; ++k) bb += (double)(scale * f[k]) * (scale * f[k]);
    double atol_sq = (double)tol * tol * bb;
    precond(n, minv, r, z);
    double rz = dotv(m, r, z);
    memcpy(p, z, m * sizeof(float));
    int it = 0;
    while (it < maxiter && rr > atol_sq) {
        spmv(n, off, col, val, fixed, p, y);
        float alpha = (float)(rz / dotv(m, p, y));
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < m; ++k) { x[k] += alpha * p[k]; r[k] -= alpha * y[k]; }
        rr = dotv(m, r, r);
        precond(n, minv, r, z);
        double rz_new = dotv(m, r, z);
        float beta = (float)(rz_new / rz);
        rz = rz_new;
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < m; ++k) p[k] = z[k] + beta * p[k];
        ++it;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            int64_t k = 3 * i + c;
            dv[k] = x[k] / scale;
            float vel = v[k] + dv[k];
            v_out[k] = fixed[i] ? 0.0f : vel;
            q_out[k] = fixed[i] ? rest[k] : q[k] + vel * dt;
        }
    return it;
}
