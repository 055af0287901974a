"""Soft-body surface contacts on the GPU (``-m gpu``) against the brute-force oracle.

Reference: ``soft_surface_contacts.py`` (SoftBodySurfaceContacts) registered by
``SolverFEM.set_soft_surface_contacts`` (solver.py:510-540) and evaluated last in
``_accumulate_forces`` (solver.py:551-589).  Two overlapping Tet4 blocks: every
surface vertex of one block inside (or within its radius of) the other is pushed
out along the pseudonormal-signed closest-point normal.  The library traverses a
BVH; the oracle tests every triangle.  Forces agree to 2e-5 of the largest entry;
a fixed-iteration substep to 1e-4 relative L2.
"""

import numpy as np
import pytest
import torch
from gpu_helpers import DEVICE, make_pair, rel_l2, rounded, tensor, to_np

from newton_solver_fem_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu

DT = 1.0 / 600.0


@pytest.fixture(autouse=True)
def _cuda(cuda_device):
    yield


def block_surface(x, tets):
    """Boundary faces of a tet mesh, oriented outward (local indices)."""
    faces = {}
    for t in tets:
        for k in range(4):
            f = [int(t[j]) for j in range(4) if j != k]
            faces.setdefault(tuple(sorted(f)), []).append((f, int(t[k])))
    out = []
    for lst in faces.values():
        if len(lst) != 1:
            continue
        (i, j, k), opp = lst[0]
        if np.dot(np.cross(x[j] - x[i], x[k] - x[i]), x[opp] - x[i]) > 0:
            j, k = k, j
        out.append((i, j, k))
    return np.asarray(out, np.int32)


def two_blocks(n=3, cell=0.02, shift=(0.055, 0.013, 0.007), **kw):
    xa, ta, ma, massa = scenes.tet_block(n, n, n, cell, (0.0, 0.0, 0.0), 1.0e5, 0.4, 1000.0)
    xb, tb, mb, massb = scenes.tet_block(n, n, n, cell, shift, 1.0e5, 0.4, 1000.0)
    na = len(xa)
    x = np.concatenate([xa, xb])
    tets = np.concatenate([ta, tb + na]).astype(np.int32)
    mats = np.concatenate([ma, mb])
    mass = np.concatenate([massa, massb])
    ranges = [(0, na), (na, len(xb))]
    tris = [block_surface(xa, ta), block_surface(xb, tb)]
    args = dict(tets=tets, tet_materials=mats, radius=0.004, gravity=(0.0, 0.0, 0.0))
    args.update(kw)
    model, solver, oracle = make_pair(x, mass, **args)
    solver.set_soft_surface_contacts(ranges, tris, ke=2.0e3, kd=50.0)
    oracle.surface = ([(s, c, t) for (s, c), t in zip(ranges, tris)], 2.0e3, 50.0)
    return model, solver, oracle


def test_surface_forces_match_brute_force_and_refit_on_update():
    model, solver, oracle = two_blocks()
    rng = np.random.default_rng(4)
    q = rounded(oracle.rest + rng.normal(0, 5e-4, oracle.rest.shape))
    v = rounded(rng.normal(0, 0.2, q.shape))
    qt, vt = tensor(q), tensor(v)
    f = solver.soft_surface_contacts.eval_forces(qt, vt)
    f2 = solver.soft_surface_contacts.eval_forces(qt, vt)
    torch.cuda.synchronize()
    assert torch.equal(f, f2)
    want = oracle.forces(q, v, terms=("surface",))["surface"]  # surfaces at the registration positions
    assert (np.abs(want).sum(1) > 0).sum() >= 8
    np.testing.assert_allclose(to_np(f), want, rtol=0, atol=2e-5 * np.abs(want).max())
    # surfaces follow an explicit refit, not the queried positions
    moved = rounded(q + (0.004, 0.0, 0.0))
    solver.soft_surface_contacts.update(tensor(moved))
    oracle.refit_surfaces(moved)
    f3 = to_np(solver.soft_surface_contacts.eval_forces(qt, vt))
    want3 = oracle.forces(q, v, terms=("surface",))["surface"]
    np.testing.assert_allclose(f3, want3, rtol=0, atol=2e-5 * np.abs(want3).max())
    assert np.abs(f3 - to_np(f)).max() > 1e-3 * np.abs(want).max()


def test_substep_with_surface_contacts_matches_oracle():
    model, solver, oracle = two_blocks(linear_solver_maxiter=10, linear_solver_tolerance=1e-30)
    rng = np.random.default_rng(9)
    q = rounded(oracle.rest + rng.normal(0, 3e-4, oracle.rest.shape))
    vel = rounded(rng.normal(0, 0.05, q.shape))
    s0, s1 = model.state(), model.state()
    s0.particle_q.copy_(tensor(q))
    s0.particle_qd.copy_(tensor(vel))
    solver.refresh_tangent(s0.particle_q)  # the first refresh refits the surfaces at q
    oracle.refresh_tangent(q)
    assert np.abs(oracle.forces(q, vel, terms=("surface",))["surface"]).max() > 0
    solver.step(s0, s1, None, None, DT)
    _, v_ref, rhs = oracle.step(q, vel, DT, fixed_iterations=10)
    assert rel_l2(to_np(s0.particle_f), rhs) < 1e-5
    assert rel_l2(to_np(solver.velocity_increment), oracle.dv) < 1e-4
    assert rel_l2(to_np(s1.particle_qd), v_ref) < 1e-4


def test_surface_registration_checks_and_adjoint_refusal():
    model, solver, _ = two_blocks(n=2)
    lib = _lib.load()
    z = torch.zeros((model.particle_count, 3), device=DEVICE)
    code = lib.fem_force_vjp(solver._handle, z.data_ptr(), z.data_ptr(), None, model.gravity.data_ptr(), z.data_ptr(),
                             z.data_ptr(), z.data_ptr(), None, None, torch.cuda.current_stream().cuda_stream)
    assert code == _lib.FEM_ERR_UNSUPPORTED
    with pytest.raises(ValueError, match="local"):
        solver.set_soft_surface_contacts([(0, 4)], [np.array([[0, 1, 9]])])
    solver.set_soft_surface_contacts([], [])  # clears
    assert float(solver.soft_surface_contacts.eval_forces(model.particle_q, z).abs().max()) == 0.0
