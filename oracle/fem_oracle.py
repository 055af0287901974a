"""CPU oracle for the SolverFEM per-substep hot path -- TEST INFRASTRUCTURE ONLY.

This module is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it.
It restates, in vectorised float64 NumPy, the reference's algorithm for the path:
Stable Neo-Hookean Tet4/Hex8 forces and approximate PSD tangent, the triplet
layout and BSR assembly of ``A = M + h^2 K~ + h C_s``, the elastic predictor,
the fixed-node projection ``PAP + I - P``, RHS normalisation, block-Jacobi and
the preconditioned CG with warm start.  Every function cites the reference file
and lines it follows (paths inside ``src/newton_solver_fem/_src/solvers/fem/``
unless stated).

Parity pinning.  The reference needs Warp 1.17 and Newton 1.7, which cannot be
installed here, so it cannot be run.  This oracle is instead pinned against the
reference's own known-answer tests (Hex8 2x3x4 box quadrature and free fall,
free fall across mass scales, the h/2 force gradient, grid volume and mass,
rigid-motion invariance, force = -grad(energy), dense-solve agreement, block
inverse scale invariance) on the reference's ASCII fixture meshes; see
``tests/test_oracle_pins.py``.  The CG iterate sequence of Warp's ``cg`` is not
pinned by the reference (only residual/tolerance semantics are), and the bits
of Warp's ``svd3`` are not pinned (only clamp behaviour), so those parts are
restated from the published methods.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

PARTICLE_FLAG_ACTIVE = 1

# ---------------------------------------------------------------------------
# Hex8 reference-element data (kernels.py:1356-1419; builder.py:101-104)
# ---------------------------------------------------------------------------

HEX_SIGNS = np.array(
    [[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]],
    dtype=np.float64,
)
HEX_GP = 0.5773502691896258  # kernels.py:1357


def hex_dN_dxi() -> np.ndarray:
    """dN_a/d(xi,eta,zeta) at Gauss point g, [8 g, 8 a, 3] (kernels.py:1362-1419)."""
    gp = HEX_SIGNS * HEX_GP  # g-th point has the signs of corner g (kernels.py:1362-1383)
    out = np.empty((8, 8, 3))
    for g in range(8):
        xi, eta, zeta = gp[g]
        for a in range(8):
            xa, ya, za = HEX_SIGNS[a]
            out[g, a] = (
                xa * (1 + ya * eta) * (1 + za * zeta) * 0.125,
                (1 + xa * xi) * ya * (1 + za * zeta) * 0.125,
                (1 + xa * xi) * (1 + ya * eta) * za * 0.125,
            )
    return out


def hex_builder_data(rest: np.ndarray, hexes: np.ndarray):
    """``inv_J0`` [H,8,3,3] and ``|det J0|`` [H,8] in float64 (builder.py:95-135)."""
    dxi = hex_dN_dxi()
    J = np.einsum("hai,gaj->hgij", rest[hexes].astype(np.float64), dxi)
    det = np.linalg.det(J)
    if np.any(det <= 1.0e-12):
        raise ValueError("Degenerate or inverted Hex8")
    return np.linalg.inv(J), np.abs(det)


def hex_shape_gradients(inv_J0: np.ndarray) -> np.ndarray:
    """Reference-config gradients ``grad_X N_a = inv_J0^T dN/dxi``, [H,8 g,8 a,3] (kernels.py:1540-1548)."""
    return np.einsum("hgji,gaj->hgai", inv_J0, hex_dN_dxi())


# ---------------------------------------------------------------------------
# Principal-stretch clamp (kernels.py:421-444)
# ---------------------------------------------------------------------------


def signed_svd(F: np.ndarray):
    """SVD with U, V proper rotations and the sign of det(F) on the last singular value.

    This is the rotation-variant convention of McAdams et al. 2011 ("Computing
    the singular value decomposition of 3x3 matrices with minimal branching and
    elementary floating point operations"), which the reference's ``wp.svd3`` call
    follows: an inverted element shows up as a negative smallest stretch.
    """
    U, S, Vt = np.linalg.svd(F)
    V = np.swapaxes(Vt, -1, -2).copy()
    U = U.copy()
    S = S.copy()
    fu = np.linalg.det(U) < 0
    U[fu, :, 2] *= -1.0
    S[fu, 2] *= -1.0
    fv = np.linalg.det(V) < 0
    V[fv, :, 2] *= -1.0
    S[fv, 2] *= -1.0
    return U, S, V


def clamp_stretch(F: np.ndarray, lo: float, hi: float) -> np.ndarray:
    """``U diag(clamp(S, lo, hi)) V^T``; identity map when a bound is negative (kernels.py:421-444).

    Matrices whose signed stretches provably lie in [lo, hi] are returned
    unchanged, which is what the clamp does to them; only the others are
    decomposed.  The test is sufficient: J > 0, ||F||_F^2 <= hi^2 bounds the
    largest stretch, and the smallest is J / (s_a s_b) >= 2 J / ||F||_F^2 >= lo.
    """
    if lo < 0.0 or hi < 0.0 or len(F) == 0:
        return F
    ic = np.sum(F * F, axis=(-2, -1))
    J = np.linalg.det(F)
    need = ~((J > 0.0) & (ic <= hi * hi) & (2.0 * J >= lo * ic))
    if not need.any():
        return F
    out = np.array(F, copy=True)
    U, S, V = signed_svd(F[need])
    S = np.maximum(np.minimum(S, hi), lo)
    out[need] = np.einsum("eij,ej,ekj->eik", U, S, V)
    return out


def clamp_active(F: np.ndarray, lo: float, hi: float) -> np.ndarray:
    """Elements whose signed stretches leave [lo, hi] (the clamp changes F)."""
    if lo < 0.0 or hi < 0.0 or len(F) == 0:
        return np.zeros(len(F), bool)
    _, S, _ = signed_svd(F)
    return np.any((S < lo) | (S > hi), axis=1)


# ---------------------------------------------------------------------------
# Force terms
# ---------------------------------------------------------------------------


def _cols(a, b, c):
    return np.stack([a, b, c], axis=-1)


def tet_forces(x, v, tets, poses, mats, lo, hi, activation=None, mu_scale=None):
    """Stable Neo-Hookean Tet4 force + Rayleigh damping (kernels.py:511-632).

    ``activation`` adds Newton's volumetric contraction term (kernels.py:484-508).
    ``mu_scale`` multiplies the shear modulus per element (the differentiable
    beam's per-element activation scale; not in the reference).
    """
    f = np.zeros_like(x, dtype=np.float64)
    if len(tets) == 0:
        return f
    mu, lam, kd = (mats[:, c].astype(np.float64) for c in range(3))
    if mu_scale is not None:
        mu = mu * mu_scale
    live = ~((mu == 0.0) & (lam == 0.0) & (kd == 0.0))  # kernels.py:545-548
    t = tets[live]
    mu, lam, kd = mu[live], lam[live], kd[live]
    Dm = poses[live].astype(np.float64)
    xs = x[t].astype(np.float64)
    vs = v[t].astype(np.float64)
    x10, x20, x30 = xs[:, 1] - xs[:, 0], xs[:, 2] - xs[:, 0], xs[:, 3] - xs[:, 0]
    v10, v20, v30 = vs[:, 1] - vs[:, 0], vs[:, 2] - vs[:, 0], vs[:, 3] - vs[:, 0]
    inv_rest_volume = np.linalg.det(Dm) * 6.0
    rest_volume = 1.0 / inv_rest_volume
    with np.errstate(divide="ignore", invalid="ignore"):
        alpha = 1.0 + mu / lam - mu / (4.0 * lam)  # kernels.py:575
    k_mu, k_lam, k_damp = mu * rest_volume, lam * rest_volume, kd * rest_volume
    F = clamp_stretch(_cols(x10, x20, x30) @ Dm, lo, hi)
    dFdt = _cols(v10, v20, v30) @ Dm
    Ic = np.sum(F * F, axis=(1, 2))
    P = F * (k_mu * (1.0 - 1.0 / (Ic + 1.0)))[:, None, None] + dFdt * k_damp[:, None, None]
    H = P @ np.swapaxes(Dm, 1, 2)
    f1, f2, f3 = H[:, :, 0], H[:, :, 1], H[:, :, 2]
    J = np.maximum(np.linalg.det(F), 0.01)  # kernels.py:608-610
    s = (inv_rest_volume / 6.0)[:, None]
    d1, d2, d3 = np.cross(x20, x30) * s, np.cross(x30, x10) * s, np.cross(x10, x20) * s
    f_volume = (J - alpha) * k_lam
    f_damp = (np.sum(d1 * v10, 1) + np.sum(d2 * v20, 1) + np.sum(d3 * v30, 1)) * k_damp
    ft = (f_volume + f_damp)[:, None]
    f1, f2, f3 = f1 + d1 * ft, f2 + d2 * ft, f3 + d3 * ft
    f0 = -(f1 + f2 + f3)
    for a, fa in enumerate((f0, f1, f2, f3)):
        np.subtract.at(f, t[:, a], fa)
    if activation is not None:
        f += tet_activation_forces(x, tets, mats, activation)
    return f


def tet_activation_forces(x, tets, mats, activation):
    """Newton's additive volumetric activation force lambda*a/6 * face crosses (kernels.py:484-508)."""
    f = np.zeros_like(x, dtype=np.float64)
    xs = x[tets].astype(np.float64)
    scale = (mats[:, 1].astype(np.float64) * np.asarray(activation, np.float64) / 6.0)[:, None]
    xa, xb, xc, xd = xs[:, 0], xs[:, 1], xs[:, 2], xs[:, 3]
    fb = scale * np.cross(xc - xa, xd - xa)
    fc = scale * np.cross(xd - xa, xb - xa)
    fd = scale * np.cross(xb - xa, xc - xa)
    np.add.at(f, tets[:, 0], fb + fc + fd)
    np.subtract.at(f, tets[:, 1], fb)
    np.subtract.at(f, tets[:, 2], fc)
    np.subtract.at(f, tets[:, 3], fd)
    return f


def _hex_F(xe, dN):
    # F = sum_a x_a (outer) grad_X N_a; absolute positions (kernels.py:1551-1560)
    return np.einsum("hai,hgaj->hgij", xe, dN)


def hex_forces(x, v, hexes, inv_J0, det_J0_w, mats, lo, hi):
    """Q1 Hex8 Stable Neo-Hookean force over the 2x2x2 Gauss rule (kernels.py:1481-1601)."""
    f = np.zeros_like(x, dtype=np.float64)
    if len(hexes) == 0:
        return f
    mu, lam, kd = (mats[:, c].astype(np.float64) for c in range(3))
    with np.errstate(divide="ignore", invalid="ignore"):
        alpha = 1.0 + mu / lam - mu / (4.0 * lam)  # kernels.py:1503 (no zero-lambda guard)
    dN = hex_shape_gradients(inv_J0.astype(np.float64))
    xe, ve = x[hexes].astype(np.float64), v[hexes].astype(np.float64)
    H = len(hexes)
    F = clamp_stretch(_hex_F(xe, dN).reshape(-1, 3, 3), lo, hi).reshape(H, 8, 3, 3)
    dFdt = _hex_F(ve, dN)
    Ic = np.sum(F * F, axis=(2, 3))
    P = F * (mu[:, None] * (1.0 - 1.0 / (Ic + 1.0)))[..., None, None] + dFdt * kd[:, None, None, None]
    J = np.maximum(np.linalg.det(F), 0.01)
    c0, c1, c2 = F[..., :, 0], F[..., :, 1], F[..., :, 2]
    cof = _cols(np.cross(c1, c2), np.cross(c2, c0), np.cross(c0, c1))
    P = P + cof * (lam[:, None] * (J - alpha[:, None]))[..., None, None]
    w = det_J0_w.astype(np.float64)
    fa = np.einsum("hg,hgij,hgaj->hai", w, P, dN)
    np.subtract.at(f, hexes.ravel(), fa.reshape(-1, 3))
    return f


def spring_forces(x, v, springs, rest, ke, kd):
    """Linear spring + damping (kernels.py:176-218)."""
    f = np.zeros_like(x, dtype=np.float64)
    if len(springs) == 0:
        return f
    i, j = springs[:, 0], springs[:, 1]
    ok = (i >= 0) & (j >= 0)
    i, j = i[ok], j[ok]
    xij = x[i].astype(np.float64) - x[j]
    vij = v[i].astype(np.float64) - v[j]
    L = np.linalg.norm(xij, axis=1)
    ok = L >= 1.0e-6
    i, j, xij, vij, L = i[ok], j[ok], xij[ok], vij[ok], L[ok]
    d = xij / L[:, None]
    c = L - rest[ok]
    fs = d * (ke[ok] * c + kd[ok] * np.sum(d * vij, 1))[:, None]
    np.subtract.at(f, i, fs)
    np.add.at(f, j, fs)
    return f


def _normalize(a):
    """Row-wise a / |a| with zero rows for |a| = 0 (Warp's normalize)."""
    n = np.linalg.norm(a, axis=-1, keepdims=True)
    return np.where(n > 0, a / np.where(n > 0, n, 1.0), 0.0)


def spring_torque_forces(x, v, springs, rest_direction, kt, kwt):
    """Bend-torque part of the torque springs: + on node j, - on node i (kernels.py:221-291)."""
    f = np.zeros_like(x, dtype=np.float64)
    if len(springs) == 0 or kt <= 0.0:
        return f
    d0 = -np.asarray(rest_direction, np.float64)
    i, j = springs[:, 0], springs[:, 1]
    xij = x[i].astype(np.float64) - x[j]
    vij = v[i].astype(np.float64) - v[j]
    L = np.linalg.norm(xij, axis=1)
    ok = (i >= 0) & (j >= 0) & (L >= 1.0e-6) & (np.linalg.norm(d0, axis=1) >= 0.5)
    d = xij / np.where(L > 0, L, 1.0)[:, None]
    theta = np.arccos(np.clip(np.sum(d * d0, 1), -1.0, 1.0))
    axis = np.cross(d0, d)
    alen = np.linalg.norm(axis, axis=1)
    ok &= alen >= 1.0e-6
    axis = axis / np.where(alen > 0, alen, 1.0)[:, None]
    d_dot = (vij - d * np.sum(d * vij, 1)[:, None]) / np.where(L > 0, L, 1.0)[:, None]
    omega = np.sum(np.cross(d, d_dot) * axis, 1)
    tau = -(kt * theta + kwt * omega) * L
    ft = np.cross(axis * tau[:, None], d) / np.where(L > 0, L, 1.0)[:, None]
    np.subtract.at(f, i[ok], ft[ok])
    np.add.at(f, j[ok], ft[ok])
    return f


def triangle_forces(x, v, tris, poses, mats):
    """Triangle membrane + area + drag/lift force (kernels.py:876-960)."""
    f = np.zeros_like(x, dtype=np.float64)
    if len(tris) == 0:
        return f
    x = x.astype(np.float64)
    v = v.astype(np.float64)
    Dm = np.asarray(poses, np.float64).reshape(-1, 2, 2)
    mats = np.asarray(mats, np.float64)
    inv_rest_area = np.linalg.det(Dm) * 2.0
    rest_area = 1.0 / inv_rest_area
    k_mu, k_lambda, k_damp = mats[:, 0] * rest_area, mats[:, 1] * rest_area, mats[:, 2] * rest_area
    k_drag, k_lift = mats[:, 3], mats[:, 4]
    i, j, k = tris[:, 0], tris[:, 1], tris[:, 2]
    x10, x20 = x[j] - x[i], x[k] - x[i]
    v10, v20 = v[j] - v[i], v[k] - v[i]
    F1 = x10 * Dm[:, 0, 0, None] + x20 * Dm[:, 1, 0, None]
    F2 = x10 * Dm[:, 0, 1, None] + x20 * Dm[:, 1, 1, None]
    dF1 = v10 * Dm[:, 0, 0, None] + v20 * Dm[:, 1, 0, None]
    dF2 = v10 * Dm[:, 0, 1, None] + v20 * Dm[:, 1, 1, None]
    Ic = np.sum(F1 * F1, 1) + np.sum(F2 * F2, 1)
    dev = (Ic - 2.0) / Ic
    P1 = F1 * (k_mu * dev)[:, None] + dF1 * k_damp[:, None]
    P2 = F2 * (k_mu * dev)[:, None] + dF2 * k_damp[:, None]
    f1 = P1 * Dm[:, 0, 0, None] + P2 * Dm[:, 0, 1, None]
    f2 = P1 * Dm[:, 1, 0, None] + P2 * Dm[:, 1, 1, None]
    n = np.cross(x10, x20)
    area = np.linalg.norm(n, axis=1) * 0.5
    c = area * inv_rest_area - 1.0
    n = _normalize(n)
    dcdq = np.cross(x20, n) * (inv_rest_area * 0.5)[:, None]
    dcdr = np.cross(n, x10) * (inv_rest_area * 0.5)[:, None]
    dcdt = np.sum(dcdq * v[j], 1) + np.sum(dcdr * v[k], 1) - np.sum((dcdq + dcdr) * v[i], 1)
    s = k_lambda * c + k_damp * dcdt
    f1 = f1 + dcdq * s[:, None]
    f2 = f2 + dcdr * s[:, None]
    f0 = f1 + f2
    vmid = (v[i] + v[j] + v[k]) * 0.3333
    vdir = _normalize(vmid)
    f_drag = vmid * (k_drag * area * np.abs(np.sum(n * vmid, 1)))[:, None]
    lift = k_lift * area * (np.pi / 2 - np.arccos(np.clip(np.sum(n * vdir, 1), -1.0, 1.0)))
    f_lift = n * (lift * np.sum(vmid * vmid, 1))[:, None]
    np.add.at(f, i, f0 - f_drag - f_lift)
    np.subtract.at(f, j, f1 + f_drag + f_lift)
    np.subtract.at(f, k, f2 + f_drag + f_lift)
    return f


def particle_contact_forces(x, v, radius, flags, ke, kd, kf, mu, cohesion):
    """Particle-particle penalty + damping + Coulomb over all pairs with d - r_i - r_j <= cohesion.

    Brute force over pairs: the neighbour set of the reference's hash-grid
    query after its filter (kernels.py:1036-1114, particle_force 1050-1076).
    """
    x = np.asarray(x, np.float64)
    v = np.asarray(v, np.float64)
    radius = np.asarray(radius, np.float64)
    active = (np.asarray(flags) & PARTICLE_FLAG_ACTIVE) != 0
    f = np.zeros_like(x)
    P = len(x)
    for lo in range(0, P, 512):
        hi = min(P, lo + 512)
        n = x[lo:hi, None, :] - x[None, :, :]
        d = np.linalg.norm(n, axis=2)
        err = d - radius[lo:hi, None] - radius[None, :]
        ok = (err <= cohesion) & (d >= 1.0e-10) & active[lo:hi, None] & active[None, :]
        ok[np.arange(hi - lo), np.arange(lo, hi)] = False
        ii, jj = np.nonzero(ok)
        if len(ii) == 0:
            continue
        nn = n[ii, jj] / d[ii, jj][:, None]
        vrel = v[lo + ii] - v[jj]
        vn = np.sum(nn * vrel, 1)
        fn = err[ii, jj] * ke + np.minimum(vn, 0.0) * kd
        vt = vrel - nn * vn[:, None]
        vs = np.linalg.norm(vt, axis=1)
        vt = np.where(vs[:, None] > 0, vt / np.where(vs > 0, vs, 1.0)[:, None], vt)
        ft = np.minimum(vs * kf, mu * np.abs(fn))
        np.add.at(f, lo + ii, -nn * fn[:, None] - vt * ft[:, None])
    return f


def soft_contact_forces(x, v, radius, count, particle, body_pos, body_vel, normal, ke, kd, kf, mu):
    """Force-based soft-rigid contacts of the first ``count`` list entries (kernels.py:1198-1261)."""
    x = np.asarray(x, np.float64)
    v = np.asarray(v, np.float64)
    f = np.zeros_like(x)
    for c in range(int(count)):
        p = int(particle[c])
        if p < 0 or p >= len(x):
            continue
        n = np.asarray(normal[c], np.float64)
        pen = radius[p] - np.dot(x[p] - body_pos[c], n)
        if not pen > 0.0:
            continue
        rel = v[p] - body_vel[c]
        vn = np.dot(rel, n)
        vt = rel - vn * n
        fn = ke * pen - kd * min(vn, 0.0)
        vt_mag = np.linalg.norm(vt)
        if vt_mag > 1.0e-6:
            ft = min(kf * vt_mag, mu * max(0.0, fn))
            f[p] += fn * n - ft * (vt / vt_mag)
        else:
            f[p] += fn * n
    return f


def closest_on_triangles(p, a, b, c):
    """Closest points of triangles (a, b, c) [n, 3] to the point p, and their feature codes
    (0 face, 1..3 edge ab, bc, ca, 4..6 vertex a, b, c): the Voronoi-region method."""
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = np.sum(ab * ap, 1), np.sum(ac * ap, 1)
    bp = p - b
    d3, d4 = np.sum(ab * bp, 1), np.sum(ac * bp, 1)
    cp = p - c
    d5, d6 = np.sum(ab * cp, 1), np.sum(ac * cp, 1)
    vc = d1 * d4 - d3 * d2
    vb = d5 * d2 - d1 * d6
    va = d3 * d6 - d5 * d4
    n = len(a)
    out = np.zeros((n, 3))
    feat = np.full(n, -1)
    done = np.zeros(n, bool)

    def take(mask, pts, code):
        m = mask & ~done
        out[m] = pts[m]
        feat[m] = code
        done[m] = True

    with np.errstate(divide="ignore", invalid="ignore"):
        take((d1 <= 0) & (d2 <= 0), a, 4)
        take((d3 >= 0) & (d4 <= d3), b, 5)
        take((vc <= 0) & (d1 >= 0) & (d3 <= 0), a + ab * (d1 / (d1 - d3))[:, None], 1)
        take((d6 >= 0) & (d5 <= d6), c, 6)
        take((vb <= 0) & (d2 >= 0) & (d6 <= 0), a + ac * (d2 / (d2 - d6))[:, None], 3)
        take((va <= 0) & ((d4 - d3) >= 0) & ((d5 - d6) >= 0),
             b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)))[:, None], 2)
        denom = 1.0 / (va + vb + vc)
        take(np.ones(n, bool), a + ab * (vb * denom)[:, None] + ac * (vc * denom)[:, None], 0)
    return out, feat


def surface_pseudonormals(x, tris):
    """Unit face normals, angle-weighted vertex pseudonormals (dict node -> normal) and edge
    pseudonormals (face normal plus the adjacent one) of a triangle surface at positions x."""
    x = np.asarray(x, np.float64)
    a, b, c = x[tris[:, 0]], x[tris[:, 1]], x[tris[:, 2]]
    fn = np.cross(b - a, c - a)
    fn = fn / np.maximum(np.linalg.norm(fn, axis=1, keepdims=True), 1e-300)

    def angle(p, q, r):
        u, w = q - p, r - p
        cosv = np.sum(u * w, 1) / (np.linalg.norm(u, axis=1) * np.linalg.norm(w, axis=1))
        return np.arccos(np.clip(cosv, -1.0, 1.0))

    vn = {}
    for k, ang in enumerate((angle(a, b, c), angle(b, c, a), angle(c, a, b))):
        for t in range(len(tris)):
            v = int(tris[t, k])
            vn[v] = vn.get(v, np.zeros(3)) + fn[t] * ang[t]
    edges = {}
    for t in range(len(tris)):
        for k in range(3):
            e = tuple(sorted((int(tris[t, k]), int(tris[t, (k + 1) % 3]))))
            edges.setdefault(e, []).append(t)
    en = np.zeros((len(tris), 3, 3))
    for t in range(len(tris)):
        for k in range(3):
            e = tuple(sorted((int(tris[t, k]), int(tris[t, (k + 1) % 3]))))
            others = [o for o in edges[e] if o != t]
            en[t, k] = fn[t] + (fn[others[0]] if others else 0.0)
    return fn, vn, en


def surface_contact_forces(q, v, radius, flags, bodies, x_surface, x_registration, ke, kd):
    """Soft-body surface contact force (soft_surface_contacts.py:62-135), by brute force over triangles.

    ``bodies`` lists (start, count, local triangles).  Surfaces sit at x_surface (the last
    refit); the search radius of a body is its bounding-box diagonal at x_registration.
    """
    q = np.asarray(q, np.float64)
    v = np.asarray(v, np.float64)
    f = np.zeros_like(q)
    geo = []
    for start, count, tris in bodies:
        tris = np.asarray(tris, np.int64).reshape(-1, 3)
        if len(tris) == 0:
            geo.append(None)
            continue
        g = tris + start
        pts = np.asarray(x_registration, np.float64)[start:start + count]
        md = float(np.linalg.norm(pts.max(0) - pts.min(0)))
        geo.append((g, md, surface_pseudonormals(x_surface, g)))
    xs = np.asarray(x_surface, np.float64)
    for b, (start, count, tris) in enumerate(bodies):
        if geo[b] is None:
            continue
        for p in np.unique(geo[b][0]):
            if (flags[p] & PARTICLE_FLAG_ACTIVE) == 0:
                continue
            for o, go in enumerate(geo):
                if o == b or go is None:
                    continue
                g, md, (fn, vn, en) = go
                pts, feat = closest_on_triangles(q[p], xs[g[:, 0]], xs[g[:, 1]], xs[g[:, 2]])
                d2 = np.sum((q[p] - pts) ** 2, 1)
                t = int(np.argmin(d2))
                if not d2[t] < md * md:
                    continue
                diff = q[p] - pts[t]
                raw = float(np.linalg.norm(diff))
                if raw < 1.0e-8:
                    continue
                ft = int(feat[t])
                pn = fn[t] if ft == 0 else (en[t, ft - 1] if ft <= 3 else vn[int(g[t, ft - 4])])
                sign = 1.0 if np.dot(diff, pn) >= 0.0 else -1.0
                n = diff / raw * sign
                pen = radius[p] - raw * sign
                if not pen > 0.0:
                    continue
                f[p] += n * (ke * pen - kd * min(float(np.dot(v[p], n)), 0.0))
    return f


def ground_forces(x, v, radius, inv_mass, flags, ke, kd, kf, mu, plane, gravity):
    """Analytic ground penalty + weight-capped Coulomb friction (kernels.py:1132-1195)."""
    x = x.astype(np.float64)
    v = v.astype(np.float64)
    n = np.asarray(plane[:3], np.float64)
    c = np.minimum(x @ n + plane[3] - radius, 0.0)
    vn = v @ n
    jn = c * ke
    jd = np.minimum(vn, 0.0) * kd
    fn = jn + jd
    vt = v - n[None] * vn[:, None]
    vs = np.linalg.norm(vt, axis=1)
    vt = np.where(vs[:, None] > 0, vt / np.where(vs > 0, vs, 1.0)[:, None], vt)
    gmag = float(np.linalg.norm(gravity))
    m = np.where(inv_mass > 0.0, 1.0 / np.maximum(inv_mass, 1e-9), 0.0)
    fn_eff = np.minimum(np.abs(fn), m * gmag)
    ft = np.minimum(vs * kf, mu * fn_eff)
    f = -n[None] * fn[:, None] - vt * ft[:, None]
    live = ((flags & PARTICLE_FLAG_ACTIVE) != 0) & (c < 0.0)
    return np.where(live[:, None], f, 0.0)


def gravity_forces(mass, flags, gravity):
    """f = m g for active particles (kernels.py:1273-1286)."""
    f = np.outer(mass.astype(np.float64), np.asarray(gravity, np.float64))
    return np.where(((flags & PARTICLE_FLAG_ACTIVE) != 0)[:, None], f, 0.0)


def damping_forces(v, mass, flags, alpha):
    """f = -alpha m v (kernels.py:1289-1307)."""
    f = -alpha * mass[:, None].astype(np.float64) * v
    return np.where(((flags & PARTICLE_FLAG_ACTIVE) != 0)[:, None], f, 0.0)


# ---------------------------------------------------------------------------
# Tangent blocks and triplets
# ---------------------------------------------------------------------------


def tet_tangent(x, tets, poses, mats, lo, hi, dt, mu_scale=None):
    """16 blocks ``h^2 (K_dev + K_vol)`` per tet, rows/cols -1 for empty material (kernels.py:635-850)."""
    T = len(tets)
    rows = np.repeat(tets, 4, axis=1).astype(np.int64)  # row of block (a, b) = node a
    cols = np.tile(tets, (1, 4)).astype(np.int64)  # col = node b
    vals = np.zeros((T, 16, 3, 3))
    if T == 0:
        return rows.reshape(-1), cols.reshape(-1), vals.reshape(-1, 3, 3)
    mu, lam = mats[:, 0].astype(np.float64), mats[:, 1].astype(np.float64)
    if mu_scale is not None:
        mu = mu * mu_scale
    empty = (mu == 0.0) & (lam == 0.0) & (mats[:, 2] == 0.0)  # kernels.py:690-700
    Dm = poses.astype(np.float64)
    inv_rest_volume = np.linalg.det(Dm) * 6.0
    degenerate = inv_rest_volume <= 0.0  # kernels.py:716-727: zero blocks, valid rows
    ok = ~empty & ~degenerate
    xs = x[tets].astype(np.float64)
    x10, x20, x30 = xs[:, 1] - xs[:, 0], xs[:, 2] - xs[:, 0], xs[:, 3] - xs[:, 0]
    with np.errstate(divide="ignore", invalid="ignore"):
        rest_volume = np.where(ok, 1.0 / np.where(ok, inv_rest_volume, 1.0), 0.0)
    k_mu, k_lam = mu * rest_volume, lam * rest_volume
    F = _cols(x10, x20, x30) @ Dm
    F[ok] = clamp_stretch(F[ok], lo, hi)
    Ic1 = np.maximum(np.sum(F * F, axis=(1, 2)) + 1.0, 1e-6)
    s = 1.0 - 1.0 / Ic1
    coef = k_mu * 2.0 / (Ic1 * Ic1)
    sv = (inv_rest_volume / 6.0)[:, None]
    d1, d2, d3 = np.cross(x20, x30) * sv, np.cross(x30, x10) * sv, np.cross(x10, x20) * sv
    dJ = np.stack([-(d1 + d2 + d3), d1, d2, d3], axis=1)  # [T,4,3]
    dm = np.swapaxes(Dm, 1, 2)  # columns = rows of Dm
    dm_rows = np.stack([-(Dm[:, 0] + Dm[:, 1] + Dm[:, 2]), Dm[:, 0], Dm[:, 1], Dm[:, 2]], axis=1)
    del dm
    Fdm = np.einsum("tij,taj->tai", F, dm_rows)
    dots = np.einsum("tai,tbi->tab", dm_rows, dm_rows)
    eye = np.eye(3)
    K = (
        (k_mu * s)[:, None, None, None, None] * dots[..., None, None] * eye
        + coef[:, None, None, None, None] * np.einsum("tai,tbj->tabij", Fdm, Fdm)
        + k_lam[:, None, None, None, None] * np.einsum("tai,tbj->tabij", dJ, dJ)
    ) * (dt * dt)
    K[~ok] = 0.0
    vals[:] = K.reshape(T, 16, 3, 3)
    rows[empty] = -1
    cols[empty] = -1
    return rows.reshape(-1), cols.reshape(-1), vals.reshape(-1, 3, 3)


def hex_tangent(x, hexes, inv_J0, det_J0_w, mats, lo, hi, dt):
    """64 PSD blocks per hex summed over the Gauss rule (kernels.py:1609-1747)."""
    Hn = len(hexes)
    rows = np.repeat(hexes, 8, axis=1).astype(np.int64)
    cols = np.tile(hexes, (1, 8)).astype(np.int64)
    if Hn == 0:
        return rows.reshape(-1), cols.reshape(-1), np.zeros((0, 3, 3))
    mu, lam = mats[:, 0].astype(np.float64), mats[:, 1].astype(np.float64)
    dN = hex_shape_gradients(inv_J0.astype(np.float64))
    xe = x[hexes].astype(np.float64)
    F = clamp_stretch(_hex_F(xe, dN).reshape(-1, 3, 3), lo, hi).reshape(Hn, 8, 3, 3)
    Ic1 = np.maximum(np.sum(F * F, axis=(2, 3)) + 1.0, 1e-6)
    s = 1.0 - 1.0 / Ic1
    coef = mu[:, None] * 2.0 / (Ic1 * Ic1)
    c0, c1, c2 = F[..., :, 0], F[..., :, 1], F[..., :, 2]
    cof = _cols(np.cross(c1, c2), np.cross(c2, c0), np.cross(c0, c1))
    Fd = np.einsum("hgij,hgaj->hgai", F, dN)
    dJ = np.einsum("hgij,hgaj->hgai", cof, dN)
    dots = np.einsum("hgai,hgbi->hgab", dN, dN)
    w = det_J0_w.astype(np.float64)
    # Gauss sums as batched products over g: [H, 24, g] @ [H, g, 24] -> [H, (a i), (b j)]
    def outer_sum(weight, G):
        G2 = G.reshape(Hn, 8, 24)
        return np.matmul(np.swapaxes(weight[:, :, None] * G2, 1, 2), G2).reshape(Hn, 8, 3, 8, 3).transpose(0, 1, 3, 2, 4)

    iso = np.einsum("hg,hgab->hab", w * mu[:, None] * s, dots)
    K = outer_sum(w * coef, Fd) + outer_sum(w * lam[:, None], dJ)
    K += iso[:, :, :, None, None] * np.eye(3)
    K *= dt * dt
    return rows.reshape(-1), cols.reshape(-1), K.reshape(-1, 3, 3)


def constant_triplets(mass, springs, ke, kd, dt):
    """Mass + spring diagonal and spring off-diagonal triplets (solver.py:1015-1060; kernels.py:141-153, 294-366)."""
    P = len(mass)
    diag = mass.astype(np.float64).copy()
    S = len(springs)
    if S:
        c = dt * kd.astype(np.float64) + dt * dt * ke.astype(np.float64)
        for col in (0, 1):
            idx = springs[:, col]
            ok = idx >= 0
            np.add.at(diag, idx[ok], c[ok])
    rows = [np.arange(P)]
    cols = [np.arange(P)]
    vals = [diag[:, None, None] * np.eye(3)]
    if S:
        off = -(dt * kd.astype(np.float64) + dt * dt * ke.astype(np.float64))
        r = np.stack([springs[:, 0], springs[:, 1]], axis=1).reshape(-1)
        cc = np.stack([springs[:, 1], springs[:, 0]], axis=1).reshape(-1)
        rows.append(r)
        cols.append(cc)
        vals.append(np.repeat(off, 2)[:, None, None] * np.eye(3))
    return np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)


def triangle_triplets(tris, poses, mats, dt):
    """Lumped triangle blocks h^2 (mu + lambda) A_rest / 3 per vertex, zero when degenerate (kernels.py:963-1012)."""
    if len(tris) == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros((0, 3, 3))
    Dm = np.asarray(poses, np.float64).reshape(-1, 2, 2)
    inv_rest_area = np.linalg.det(Dm) * 2.0
    ok = inv_rest_area > 0.0
    rest_area = np.where(ok, 1.0 / np.where(ok, inv_rest_area, 1.0), 0.0)
    mats = np.asarray(mats, np.float64)
    d = np.where(ok, dt * dt * (mats[:, 0] * rest_area + mats[:, 1] * rest_area) / 3.0, 0.0)
    rows = np.asarray(tris, np.int64).reshape(-1)
    return rows, rows.copy(), np.repeat(d, 3)[:, None, None] * np.eye(3)


def assemble_bsr(rows, cols, vals, n):
    """COO -> BSR with sorted columns, duplicates summed, negative indices dropped.

    Restates the behaviour the reference relies on from Warp's
    ``bsr_set_from_triplets(prune_numerical_zeros=False)`` (solver.py:677-683;
    the pattern is pinned by tests/test_solver.py:542-545).
    """
    ok = (rows >= 0) & (cols >= 0)
    rows, cols, vals = rows[ok], cols[ok], vals[ok]
    key = rows.astype(np.int64) * n + cols
    order = np.argsort(key, kind="stable")
    key = key[order]
    uniq, start = np.unique(key, return_index=True)
    summed = np.add.reduceat(vals[order], start, axis=0) if len(key) else np.zeros((0, 3, 3))
    r = (uniq // n).astype(np.int64)
    c = (uniq % n).astype(np.int32)
    offsets = np.zeros(n + 1, np.int64)
    np.add.at(offsets, r + 1, 1)
    offsets = np.cumsum(offsets)
    return offsets, c, summed


def bsr_to_scipy(offsets, columns, values, n):
    return sp.bsr_matrix((values, columns, offsets), shape=(3 * n, 3 * n))


def dense(offsets, columns, values, n):
    out = np.zeros((3 * n, 3 * n))
    for row in range(n):
        for k in range(offsets[row], offsets[row + 1]):
            c = columns[k]
            out[3 * row : 3 * row + 3, 3 * c : 3 * c + 3] += values[k]
    return out


# ---------------------------------------------------------------------------
# Preconditioner, predictor, normalisation, CG
# ---------------------------------------------------------------------------


def inverse_diagonal_block(blocks: np.ndarray, dtype=np.float64) -> np.ndarray:
    """Scale-normalised 3x3 inverse with point-Jacobi fallback (kernels.py:1817-1833)."""
    blocks = np.asarray(blocks, dtype)
    out = np.zeros_like(blocks)
    scale = np.max(np.abs(np.diagonal(blocks, axis1=1, axis2=2)), axis=1)
    good = np.zeros(len(blocks), bool)
    pos = scale > 0
    if np.any(pos):
        nrm = blocks[pos] / scale[pos, None, None]
        tr = np.trace(nrm, axis1=1, axis2=2) / dtype(3.0)
        det = np.linalg.det(nrm)
        ok = (tr > 0) & (np.abs(det) > dtype(1.0e-9) * tr * tr * tr)
        idx = np.nonzero(pos)[0][ok]
        out[idx] = np.linalg.inv(nrm[ok]) / scale[idx, None, None]
        good[idx] = True
    bad = ~good
    if np.any(bad):
        d = np.diagonal(blocks[bad], axis1=1, axis2=2)
        rec = np.where(d > 0, 1.0 / np.where(d > 0, d, 1.0), 1.0)
        out[bad] = rec[:, :, None] * np.eye(3)
    return out


def block_jacobi(offsets, columns, values, n):
    """Minv[i] = inverse_diagonal_block(A_ii), identity when the row has no diagonal (kernels.py:1836-1849)."""
    diag = np.tile(np.eye(3), (n, 1, 1))
    for_row = np.repeat(np.arange(n), np.diff(offsets))
    hit = columns == for_row
    diag[for_row[hit]] = values[hit]
    return inverse_diagonal_block(diag)


def point_jacobi(offsets, columns, values, n):
    """Inverse of the scalar diagonal, 1 where it is zero (Warp ``preconditioner(A, "diag")``)."""
    out = np.zeros((n, 3, 3))
    for_row = np.repeat(np.arange(n), np.diff(offsets))
    hit = columns == for_row
    d = np.ones((n, 3))
    d[for_row[hit]] = np.diagonal(values[hit], axis1=1, axis2=2)
    out[:, [0, 1, 2], [0, 1, 2]] = np.where(d == 0, 1.0, 1.0 / np.where(d == 0, 1.0, d))
    return out


def elastic_predictor(offsets, columns, values, v):
    """``correction_i = sum_j A_ij (v_j - v_i)`` (implicit_predictor.py:9-23)."""
    n = len(offsets) - 1
    for_row = np.repeat(np.arange(n), np.diff(offsets))
    diff = v[columns].astype(np.float64) - v[for_row]
    contrib = np.einsum("kij,kj->ki", values, diff)
    out = np.zeros((n, 3))
    np.add.at(out, for_row, contrib)
    return out


def spring_damping_restore(springs, kd, dt, v, rhs):
    """rhs_a += h d (v_a - v_b), rhs_b -= ... (implicit_predictor.py:26-41)."""
    if len(springs) == 0:
        return rhs
    a, b = springs[:, 0], springs[:, 1]
    ok = (a >= 0) & (b >= 0)
    corr = dt * kd[ok, None].astype(np.float64) * (v[a[ok]].astype(np.float64) - v[b[ok]])
    np.add.at(rhs, a[ok], corr)
    np.subtract.at(rhs, b[ok], corr)
    return rhs


def rhs_scale(maximum: float) -> float:
    """RHS normalisation factor (kernels.py:1785-1793)."""
    if 0.0 < maximum < 1.0e-12:
        return min(1.0 / maximum, 1.0e30)
    return 1.0


def pcg(apply_A, apply_M, b, x, tol, maxiter):
    """Preconditioned CG with warm start, ``atol = 0`` and a relative stop.

    Restates the semantics the reference relies on from Warp's ``cg`` (solver.py:1219-1252):
    stop once ``||r||^2 <= tol^2 ||b||^2`` (unpreconditioned residual),
    at most ``maxiter`` updates, iterate frozen after convergence.
    Returns (x, iterations, ||r||^2, ||b||^2).
    """
    x = x.copy()
    r = b - apply_A(x)
    rr = float(np.dot(r.ravel(), r.ravel()))
    bb = float(np.dot(b.ravel(), b.ravel()))
    atol_sq = tol * tol * bb
    z = apply_M(r)
    rz = float(np.dot(r.ravel(), z.ravel()))
    p = z.copy()
    it = 0
    while it < maxiter and rr > atol_sq:
        Ap = apply_A(p)
        pAp = float(np.dot(p.ravel(), Ap.ravel()))
        alpha = rz / pAp
        x += alpha * p
        r -= alpha * Ap
        rr = float(np.dot(r.ravel(), r.ravel()))
        z = apply_M(r)
        rz_new = float(np.dot(r.ravel(), z.ravel()))
        beta = rz_new / rz
        rz = rz_new
        p = z + beta * p
        it += 1
    return x, it, rr, bb


# ---------------------------------------------------------------------------
# Whole solver (solver.py:212-415, 942-1002, 1254-1351)
# ---------------------------------------------------------------------------


class OracleFEM:
    """CPU restatement of ``SolverFEM`` on the hot-path configuration (CG, block Jacobi)."""

    def __init__(
        self,
        x,
        mass,
        *,
        tets=None,
        tet_poses=None,
        tet_materials=None,
        hexes=None,
        hex_inv_J0=None,
        hex_det_J0_w=None,
        hex_materials=None,
        springs=None,
        spring_rest=None,
        spring_ke=None,
        spring_kd=None,
        radius=None,
        flags=None,
        gravity=(0.0, 0.0, -9.81),
        dt=1.0 / 60.0,
        min_stretch=0.05,
        max_stretch=20.0,
        ground_plane=None,
        ground_ke=1.0e5,
        ground_kd=1.0e2,
        ground_kf=1.0e3,
        ground_mu=0.5,
        linear_damping=0.0,
        fixed=None,
        maxiter=50,
        tolerance=1.0e-2,
        preconditioner="block_diag",
        mu_scale=None,
        scene_offsets=None,
        tris=None,
        tri_poses=None,
        tri_materials=None,
        spring_rest_direction=None,
        torque_stiffness=0.0,
        torque_damping=0.0,
        particle_contact=None,
        soft_contact=(1.0e3, 10.0, 1.0e3, 0.5),
        surface=None,
    ):
        """``particle_contact`` = (ke, kd, kf, mu, cohesion) enables the particle-particle term;
        ``surface`` = (bodies, ke, kd) registers surface contacts at the construction positions."""
        self.rest = np.asarray(x, np.float64).copy()
        self.n = len(self.rest)
        self.mass = np.asarray(mass, np.float64)
        self.inv_mass = np.where(self.mass > 0, 1.0 / np.where(self.mass > 0, self.mass, 1.0), 0.0)
        z4, z8 = np.zeros((0, 4), np.int32), np.zeros((0, 8), np.int32)
        self.tets = z4 if tets is None else np.asarray(tets, np.int64)
        self.tet_poses = np.zeros((0, 3, 3)) if tet_poses is None else np.asarray(tet_poses)
        self.tet_materials = np.zeros((0, 3)) if tet_materials is None else np.asarray(tet_materials)
        self.hexes = z8 if hexes is None else np.asarray(hexes, np.int64)
        self.hex_inv_J0 = hex_inv_J0
        self.hex_det_J0_w = hex_det_J0_w
        self.hex_materials = np.zeros((0, 3)) if hex_materials is None else np.asarray(hex_materials)
        self.springs = np.zeros((0, 2), np.int64) if springs is None else np.asarray(springs, np.int64)
        S = len(self.springs)
        self.spring_rest = np.zeros(S) if spring_rest is None else np.asarray(spring_rest, np.float64)
        self.spring_ke = np.zeros(S) if spring_ke is None else np.asarray(spring_ke, np.float64)
        self.spring_kd = np.zeros(S) if spring_kd is None else np.asarray(spring_kd, np.float64)
        self.radius = np.zeros(self.n) if radius is None else np.broadcast_to(np.asarray(radius, np.float64), (self.n,))
        self.flags = np.ones(self.n, np.int32) if flags is None else np.asarray(flags, np.int32)
        self.gravity = np.asarray(gravity, np.float64)
        self.dt = float(dt)
        self.min_stretch, self.max_stretch = float(min_stretch), float(max_stretch)
        self.ground_plane = None if ground_plane is None else np.asarray(ground_plane, np.float64)
        self.ground = (ground_ke, ground_kd, ground_kf, ground_mu)
        self.linear_damping = float(linear_damping)
        self.fixed = np.zeros(0, np.int64) if fixed is None else np.unique(np.asarray(fixed, np.int64))
        self.fixed_mask = np.zeros(self.n, bool)
        self.fixed_mask[self.fixed] = True
        self.maxiter, self.tolerance = int(maxiter), float(tolerance)
        self.preconditioner = preconditioner
        self.mu_scale = mu_scale
        self.scene_offsets = (
            np.array([0, self.n], np.int64) if scene_offsets is None else np.asarray(scene_offsets, np.int64)
        )
        self.tris = np.zeros((0, 3), np.int64) if tris is None else np.asarray(tris, np.int64).reshape(-1, 3)
        self.tri_poses = np.zeros((0, 2, 2)) if tri_poses is None else np.asarray(tri_poses, np.float64)
        self.tri_materials = np.zeros((0, 5)) if tri_materials is None else np.asarray(tri_materials, np.float64)
        self.spring_rest_direction = None if spring_rest_direction is None else \
            np.asarray(spring_rest_direction, np.float64)
        self.torque = (float(torque_stiffness), float(torque_damping))
        self.particle_contact = particle_contact
        self.soft_contact = soft_contact
        self.surface = surface
        self.surface_x = self.rest.copy()  # surfaces refit at registration
        self.dv = np.zeros((self.n, 3))
        self.last_iterations = []
        self.last_rr_bb = []
        self._assemble(self.rest, self.dt)

    # -- assembly -----------------------------------------------------------
    def triplets(self, q, dt):
        """All triplets in the reference layout [P | 2S | 3Tri | 16T | 64H] (solver.py:312-321)."""
        parts = [constant_triplets(self.mass, self.springs, self.spring_ke, self.spring_kd, dt)]
        parts.append(triangle_triplets(self.tris, self.tri_poses, self.tri_materials, dt))
        parts.append(
            tet_tangent(q, self.tets, self.tet_poses, self.tet_materials, self.min_stretch, self.max_stretch, dt,
                        self.mu_scale)
        )
        if len(self.hexes):
            parts.append(
                hex_tangent(q, self.hexes, self.hex_inv_J0, self.hex_det_J0_w, self.hex_materials, self.min_stretch,
                            self.max_stretch, dt)
            )
        rows = np.concatenate([p[0] for p in parts])
        cols = np.concatenate([p[1] for p in parts])
        vals = np.concatenate([p[2] for p in parts])
        return rows, cols, vals

    def _assemble(self, q, dt):
        self.offsets, self.columns, self.values = assemble_bsr(*self.triplets(q, dt), self.n)
        if self.preconditioner == "block_diag":
            self.minv = block_jacobi(self.offsets, self.columns, self.values, self.n)
        else:
            self.minv = point_jacobi(self.offsets, self.columns, self.values, self.n)
        self._A = bsr_to_scipy(self.offsets, self.columns, self.values, self.n).tocsr()

    def refit_surfaces(self, q):
        """Surfaces take positions q (SoftBodySurfaceContacts.update, soft_surface_contacts.py:226-237)."""
        self.surface_x = np.asarray(q, np.float64).copy()

    def refresh_tangent(self, q, dt=None):
        """Refresh the tangent at q; a dt change clears the warm start (solver.py:769-857).  The first
        refresh also refits the surfaces (solver.py:824-827 through _rebuild_element_blocks 669-670)."""
        dt = self.dt if dt is None else float(dt)
        q = np.asarray(q, np.float64).copy()
        q[self.fixed] = self.rest[self.fixed]
        if not getattr(self, "_refreshed", False):
            self._refreshed = True
            self.refit_surfaces(q)
        if dt != self.dt:
            self.dv[:] = 0.0
        self._assemble(q, dt)
        self.dt = dt
        return q

    def dense(self):
        return dense(self.offsets, self.columns, self.values, self.n)

    # -- forces --------------------------------------------------------------
    TERMS = ("spring", "tet", "hex", "tri", "particle", "ground", "soft_contact", "gravity", "damping", "surface")

    def forces(self, q, v, *, activation=None, terms=TERMS, contacts=None):
        """Per-term forces in the reference's accumulation order (solver.py:571-582).

        ``contacts`` = (count, particle, body_pos, body_vel, normal) NumPy arrays."""
        out = {}
        if "spring" in terms:
            out["spring"] = spring_forces(q, v, self.springs, self.spring_rest, self.spring_ke, self.spring_kd)
            if self.spring_rest_direction is not None and self.torque[0] > 0.0:
                out["spring"] += spring_torque_forces(q, v, self.springs, self.spring_rest_direction, *self.torque)
        if "tet" in terms:
            out["tet"] = tet_forces(q, v, self.tets, self.tet_poses, self.tet_materials, self.min_stretch,
                                    self.max_stretch, activation, self.mu_scale)
        if "hex" in terms:
            out["hex"] = hex_forces(q, v, self.hexes, self.hex_inv_J0, self.hex_det_J0_w, self.hex_materials,
                                    self.min_stretch, self.max_stretch) if len(self.hexes) else np.zeros((self.n, 3))
        if "tri" in terms:
            out["tri"] = triangle_forces(q, v, self.tris, self.tri_poses, self.tri_materials)
        if "particle" in terms:
            out["particle"] = np.zeros((self.n, 3)) if self.particle_contact is None else \
                particle_contact_forces(q, v, self.radius, self.flags, *self.particle_contact)
        if "soft_contact" in terms:
            out["soft_contact"] = np.zeros((self.n, 3)) if contacts is None else \
                soft_contact_forces(q, v, self.radius, *contacts, *self.soft_contact)
        if "ground" in terms:
            if self.ground_plane is None:
                out["ground"] = np.zeros((self.n, 3))
            else:
                ke, kd, kf, mu = self.ground
                out["ground"] = ground_forces(q, v, self.radius, self.inv_mass, self.flags, ke, kd, kf, mu,
                                              self.ground_plane, self.gravity)
        if "gravity" in terms:
            out["gravity"] = gravity_forces(self.mass, self.flags, self.gravity)
        if "damping" in terms:
            out["damping"] = damping_forces(v, self.mass, self.flags, self.linear_damping) if self.linear_damping > 0 \
                else np.zeros((self.n, 3))
        if "surface" in terms:
            out["surface"] = np.zeros((self.n, 3)) if self.surface is None else surface_contact_forces(
                q, v, self.radius, self.flags, self.surface[0], self.surface_x, self.rest, *self.surface[1:])
        return out

    # -- step ----------------------------------------------------------------
    def apply_A_projected(self, x):
        y = (self._A @ x.reshape(-1)).reshape(-1, 3)
        if len(self.fixed):
            xf = x.copy()
            xf[self.fixed] = 0.0
            y = (self._A @ xf.reshape(-1)).reshape(-1, 3)
            y[self.fixed] = x[self.fixed]
        return y

    def apply_M(self, r):
        return np.einsum("nij,nj->ni", self.minv, r)

    def step(self, q, v, dt, *, external=None, activation=None, fixed_iterations=None, contacts=None):
        """One substep: returns (q_out, v_out, rhs) (solver.py:942-1002, 1254-1351).

        ``fixed_iterations`` runs exactly that many CG updates (tolerance 0),
        the reference semantics used for iterate-level parity.
        """
        q = np.asarray(q, np.float64).copy()
        v = np.asarray(v, np.float64).copy()
        q[self.fixed] = self.rest[self.fixed]  # fixed_particles.py:11-15
        v[self.fixed] = 0.0
        terms = self.forces(q, v, activation=activation, contacts=contacts)
        f = np.zeros((self.n, 3))
        for key in self.TERMS:
            f += dt * terms[key]
        if external is not None:
            f += dt * np.asarray(external, np.float64)
        rhs = f - elastic_predictor(self.offsets, self.columns, self.values, v)
        rhs = spring_damping_restore(self.springs, self.spring_kd, dt, v, rhs)
        rhs[self.fixed] = 0.0  # fixed_particles.py:159-160
        dv = self.dv.copy()
        dv[self.fixed] = 0.0
        self.last_iterations, self.last_rr_bb = [], []
        out_dv = np.zeros_like(dv)
        for s in range(len(self.scene_offsets) - 1):
            lo, hi = self.scene_offsets[s], self.scene_offsets[s + 1]
            sl = slice(lo, hi)
            maximum = float(np.max(np.abs(rhs[sl]))) if hi > lo else 0.0
            scale = rhs_scale(maximum)
            b = np.zeros_like(rhs)
            b[sl] = scale * rhs[sl]
            x0 = np.zeros_like(rhs)
            if maximum != 0.0:
                x0[sl] = scale * dv[sl]

            def A_s(p, sl=sl):
                full = np.zeros_like(rhs)
                full[sl] = p[sl]
                y = self.apply_A_projected(full)
                out = np.zeros_like(rhs)
                out[sl] = y[sl]
                return out

            tol = 0.0 if fixed_iterations is not None else self.tolerance
            maxiter = self.maxiter if fixed_iterations is None else fixed_iterations
            x, it, rr, bb = pcg(A_s, self.apply_M, b, x0, tol, maxiter)
            out_dv[sl] = x[sl] / scale
            self.last_iterations.append(it)
            self.last_rr_bb.append((rr, bb))
        self.dv = out_dv
        v_out = v + self.dv
        q_out = q + v_out * dt
        q_out[self.fixed] = self.rest[self.fixed]
        v_out[self.fixed] = 0.0
        return q_out, v_out, rhs
