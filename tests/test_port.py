"""The C/OpenMP CPU port (the timed CPU baseline) agrees with the float64 NumPy oracle (no GPU)."""

import numpy as np
import pytest

from newton_solver_fem_gb300 import scenes
from oracle import fem_oracle as O
from oracle import fem_port


def _pair(sc, **kw):
    x = sc.x.astype(np.float32).astype(np.float64)
    m = sc.mass.astype(np.float32).astype(np.float64)
    common = dict(gravity=sc.gravity, dt=sc.dt, ground_plane=sc.ground_plane, fixed=sc.fixed if len(sc.fixed) else None)
    common.update(kw)
    ke, kd, kf, mu = sc.ground
    args = {}
    if len(sc.tets):
        args.update(tets=sc.tets, tet_poses=scenes.tet_poses(x, sc.tets), tet_materials=sc.tet_materials)
    if len(sc.hexes):
        inv, det = O.hex_builder_data(x, sc.hexes)
        args.update(hexes=sc.hexes, hex_inv_J0=inv.astype(np.float32), hex_det_J0_w=det.astype(np.float32),
                    hex_materials=sc.hex_materials)
    if len(sc.springs):
        rest = np.linalg.norm(x[sc.springs[:, 0]] - x[sc.springs[:, 1]], axis=1).astype(np.float32)
        args.update(springs=sc.springs, spring_rest=rest, spring_ke=sc.spring_ke, spring_kd=sc.spring_kd)
    port = fem_port.PortFEM(x, m, ground=sc.ground, **args, **common)
    oracle = O.OracleFEM(x, m, ground_ke=ke, ground_kd=kd, ground_kf=kf, ground_mu=mu, **args, **common)
    return x, port, oracle


def _jittered_in_contact():
    """Jittered Tet4 4^3 block with edge springs, lowered so its bottom layer presses into the ground, moving."""
    sc = scenes.tet_jittered_48(n=4)
    sc.x = sc.x - (0.0, 0.0, 0.203)
    sc.velocity = np.random.default_rng(11).normal(0.0, 0.05, sc.x.shape).astype(np.float32)
    return sc


@pytest.mark.parametrize("make", [scenes.tet_cantilever, lambda: scenes.hex_block_64(n=4), _jittered_in_contact])
def test_port_matches_oracle(make):
    sc = make()
    x, port, oracle = _pair(sc)
    np.testing.assert_array_equal(port.offsets, oracle.offsets)
    np.testing.assert_array_equal(port.columns, oracle.columns)
    np.testing.assert_allclose(port.values.reshape(-1, 3, 3), oracle.values, rtol=0,
                               atol=1e-5 * np.abs(oracle.values).max())
    v0 = np.zeros_like(x) if sc.velocity is None else sc.velocity.astype(np.float64)
    K = 12
    port.tol, port.maxiter = 1e-30, K
    _, v_port, rhs_port = port.step(x, v0, sc.dt)
    _, v_ref, rhs_ref = oracle.step(x, v0, sc.dt, fixed_iterations=K)
    assert port.last_iterations == K
    assert np.linalg.norm(port.dv - oracle.dv) / np.linalg.norm(oracle.dv) < 1e-4
    # float32 rest-state elastic forces carry ~1e-7 rounding noise where float64 gives zero
    assert np.linalg.norm(rhs_port - rhs_ref) / np.linalg.norm(rhs_ref) < 5e-4
    assert fem_port.threads() >= 1
