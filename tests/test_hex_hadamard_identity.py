"""The Walsh-Hadamard identities the Hex8 force kernel uses, checked in float64 against the
reference's Gauss table (oracle.hex_dN_dxi, kernels.py:1362-1419), on the host.

In VTK order node a (bits a0 a1 a2) has the signs s_x = (a0 xor a1) ? +1 : -1, s_y = a1 ? +1 : -1,
s_z = a2 ? +1 : -1.  With H_m = sum_a (-1)^popcount(a & m) v_a (the butterfly over the 8 lanes):
* dx/dxi = (-H3 + eta H1 + zeta H7 - eta zeta H5) / 8 and likewise for eta and zeta;
* the corner force sum_g PJ_g dN_a/dxi(g) comes from the butterfly of PJ over the points."""

import numpy as np

from oracle import fem_oracle as O

GP = 0.5773502691896258


def _signs(a):
    return (1.0 if ((a ^ (a >> 1)) & 1) else -1.0, 1.0 if a & 2 else -1.0, 1.0 if a & 4 else -1.0)


def _wht(values):
    """values[a, ...] -> H[m, ...] = sum_a (-1)^popcount(a & m) values[a, ...]."""
    chi = np.array([[(-1.0) ** bin(a & m).count("1") for a in range(8)] for m in range(8)])
    return np.tensordot(chi, values, axes=(1, 0))


def test_vtk_signs_match_the_reference_table_ordering():
    assert np.array_equal(np.array([_signs(a) for a in range(8)]), O.HEX_SIGNS)


def test_shape_derivatives_from_hadamard_coefficients():
    rng = np.random.default_rng(3)
    x = rng.normal(size=(8, 3))
    table = O.hex_dN_dxi()  # [g, a, axis]
    H = _wht(x)  # [m, component]
    for g in range(8):
        sx, sy, sz = _signs(g)
        xi, eta, zeta = sx * GP, sy * GP, sz * GP
        direct = np.einsum("ai,ak->ik", x, table[g])  # dx_i/dxi_k
        d0 = (-H[3] + eta * H[1] + zeta * H[7] - eta * zeta * H[5]) / 8
        d1 = (-H[2] + xi * H[1] + zeta * H[6] - xi * zeta * H[5]) / 8
        d2 = (-H[4] + xi * H[7] + eta * H[6] - xi * eta * H[5]) / 8
        np.testing.assert_allclose(np.stack([d0, d1, d2], axis=1), direct, rtol=1e-12, atol=1e-12)


def test_corner_forces_from_the_point_butterfly():
    rng = np.random.default_rng(4)
    PJ = rng.normal(size=(8, 3, 3))  # P inv_J0^T w at each point
    table = O.hex_dN_dxi()
    direct = np.einsum("gik,gak->ai", PJ, table)  # f_a = sum_g PJ_g dN_a/dxi(g)
    W = _wht(PJ) / 8  # the 1/8 the kernel folds into its scaled inverse Jacobian
    for a in range(8):
        sx, sy, sz = _signs(a)
        cx, cy, cz = -GP * sx, -GP * sy, -GP * sz
        cyz, cxz, cxy = GP * GP * sy * sz, GP * GP * sx * sz, GP * GP * sx * sy
        f = np.empty(3)
        for i in range(3):
            t0 = W[0][i, 0] + cy * W[2][i, 0] + cz * W[4][i, 0] + cyz * W[6][i, 0]
            t1 = W[0][i, 1] + cx * W[3][i, 1] + cz * W[4][i, 1] + cxz * W[7][i, 1]
            t2 = W[0][i, 2] + cx * W[3][i, 2] + cy * W[2][i, 2] + cxy * W[1][i, 2]
            f[i] = sx * t0 + sy * t1 + sz * t2
        np.testing.assert_allclose(f, direct[a], rtol=1e-12, atol=1e-12)
