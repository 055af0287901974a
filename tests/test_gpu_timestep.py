"""Timestep changes on the GPU (``-m gpu``): the behaviour the reference pins in
``tests/test_solver_timestep.py``.  ``refresh_tangent(q, dt)`` with a new dt
rebuilds the dt-dependent constant blocks and the element blocks in the
existing storage, so the matrix and a step equal those of a solver built fresh
at that dt; only the warm start is discarded; invalid timesteps are rejected
without changing the solver; and the differentiable step refuses a dt other
than the assembled one.
"""

import numpy as np
import pytest
import torch
from gpu_helpers import mixed_model, tensor, to_np

from newton_solver_fem_gb300 import SolverFEM
from newton_solver_fem_gb300.adjoint import DifferentiableSolver

pytestmark = pytest.mark.gpu

DT = 0.002


@pytest.fixture(autouse=True)
def _cuda(cuda_device):
    yield


def make(model, fixed, dt=DT):
    return SolverFEM(model, dt=dt, solver_type="cg", preconditioner_type="block_diag", self_contact_ke=0.0,
                     linear_solver_tolerance=1.0e-6, linear_solver_maxiter=500, fixed_particle_indices=fixed)


def test_matrix_and_step_match_fresh_solvers_across_timestep_changes():
    model, fixed, rng = mixed_model(seed=21)
    actual = make(model, fixed)
    state = model.state()
    state.particle_q.add_(tensor(rng.normal(0, 1.0e-3, tuple(state.particle_q.shape))))
    load = tensor(np.linspace(-0.01, 0.02, state.particle_q.numel()).reshape(-1, 3))
    dv_ptr = actual.velocity_increment.data_ptr()
    for dt in (DT, DT / 2, DT):
        actual.refresh_tangent(state.particle_q, dt)
        assert actual.dt == dt
        reference = make(model, fixed, dt)
        reference.refresh_tangent(state.particle_q)
        np.testing.assert_allclose(actual.A_bsr.dense(), reference.A_bsr.dense(), rtol=1e-6, atol=1e-9)
        np.testing.assert_allclose(to_np(actual._pc_inv_diag), to_np(reference._pc_inv_diag), rtol=1e-6, atol=1e-6)
        assert actual.velocity_increment.data_ptr() == dv_ptr  # storage kept
        actual.velocity_increment.zero_()
        a_in, a_out, r_in, r_out = model.state(), model.state(), model.state(), model.state()
        for s in (a_in, r_in):
            s.particle_q.copy_(state.particle_q)
            s.particle_qd.copy_(state.particle_qd)
        actual.step(a_in, a_out, None, None, dt, external_forces=load)
        reference.step(r_in, r_out, None, None, dt, external_forces=load)
        np.testing.assert_allclose(to_np(a_in.particle_f), to_np(r_in.particle_f), rtol=1e-6, atol=1e-9)
        np.testing.assert_allclose(to_np(a_out.particle_q), to_np(r_out.particle_q), rtol=1e-6, atol=1e-8)
        np.testing.assert_allclose(to_np(a_out.particle_qd), to_np(r_out.particle_qd), rtol=2e-5, atol=1e-7)
        np.testing.assert_array_equal(to_np(a_out.particle_q)[fixed], to_np(model.particle_q)[fixed])
        np.testing.assert_array_equal(to_np(a_out.particle_qd)[fixed], 0.0)
        actual.refresh_tangent(state.particle_q)  # an omitted dt keeps the assembled one
        assert actual.dt == dt


def test_changed_timestep_discards_only_the_warm_start():
    model, fixed, rng = mixed_model(seed=22)
    solver = make(model, fixed)
    state = model.state()
    q0, v0 = to_np(state.particle_q).copy(), to_np(state.particle_qd).copy()
    solver.velocity_increment.fill_(0.02)
    solver.refresh_tangent(state.particle_q)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(to_np(solver.velocity_increment), np.float32(0.02))
    solver.refresh_tangent(state.particle_q, DT / 2)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(to_np(solver.velocity_increment), 0.0)
    np.testing.assert_array_equal(to_np(state.particle_q), q0)
    np.testing.assert_array_equal(to_np(state.particle_qd), v0)


@pytest.mark.parametrize("bad", [0.0, -1.0, float("nan"), float("inf")])
def test_invalid_timestep_is_rejected_without_change(bad):
    model, fixed, _ = mixed_model(seed=23)
    solver = make(model, fixed)
    before = solver.A_bsr.dense()
    with pytest.raises(ValueError):
        solver.refresh_tangent(model.particle_q, bad)
    assert solver.dt == DT
    np.testing.assert_array_equal(solver.A_bsr.dense(), before)


def test_differentiable_step_requires_the_assembled_timestep():
    model, fixed, _ = mixed_model(seed=24)
    solver = make(model, fixed)
    diff = DifferentiableSolver(solver)
    q, v = model.particle_q.clone(), model.particle_qd.clone()
    with pytest.raises(ValueError, match="Differentiable dt"):
        diff.step(q, v, DT / 2)
    q1, v1 = diff.step(q, v, DT)
    assert torch.isfinite(q1).all() and torch.isfinite(v1).all()
