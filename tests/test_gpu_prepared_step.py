"""Prepared affine step on the GPU (``-m gpu``): the behaviour the reference pins in
``tests/test_fem_prepared_step.py`` — parity with ``step`` on mixed elements with
damping, springs, fixed supports and a load; operator, preconditioner, diagonal
blocks and RHS affinity against the exported matrix; ownership of the prepared
input and storage reuse; invalidation by a timestep change; argument checks;
and CUDA-graph replay.  Solves run to a tight tolerance, so warm starts do not
matter and the increments agree to solver precision.
"""

import numpy as np
import pytest
import torch
from gpu_helpers import DEVICE, mixed_model, tensor, to_np

from newton_solver_fem_gb300 import PreparedFEMStep, SolverFEM

pytestmark = pytest.mark.gpu

DT = 1.0 / 600.0


@pytest.fixture(autouse=True)
def _cuda(cuda_device):
    yield


def solver_for(model, fixed, **kw):
    args = dict(dt=DT, solver_type="cg", preconditioner_type="block_diag", self_contact_ke=0.0,
                linear_solver_tolerance=1.0e-6, linear_solver_maxiter=500, fixed_particle_indices=fixed)
    args.update(kw)
    return SolverFEM(model, **args)


def perturbed_state(model, rng):
    s = model.state()
    s.particle_q.add_(tensor(rng.normal(0, 1.5e-3, tuple(s.particle_q.shape))))
    return s


def copy_state(model, s):
    c = model.state()
    c.particle_q.copy_(s.particle_q)
    c.particle_qd.copy_(s.particle_qd)
    return c


def test_prepared_solve_and_reconstruct_match_step():
    model, fixed, rng = mixed_model()
    solver = solver_for(model, fixed)
    current = perturbed_state(model, rng)
    solver.refresh_tangent(current.particle_q)
    before = to_np(current.particle_q)
    prepared = solver.prepare_step(current, None, None, DT)
    np.testing.assert_array_equal(to_np(current.particle_q), before)  # the input is copied, not restored in place
    for k in range(3):
        load = tensor(rng.normal(0, 0.2, tuple(current.particle_q.shape)))
        rhs = prepared.rhs(load)
        dv = prepared.solve(rhs).clone()
        result = model.state()
        prepared.reconstruct(dv, result)
        ref_in, ref_out = copy_state(model, current), model.state()
        solver.step(ref_in, ref_out, None, None, DT, external_forces=load)
        rhs_ref = to_np(ref_in.particle_f)
        np.testing.assert_allclose(to_np(rhs), rhs_ref, rtol=2e-6, atol=2e-6 * np.abs(rhs_ref).max())
        dv_ref = to_np(solver.velocity_increment)
        np.testing.assert_allclose(to_np(dv), dv_ref, rtol=0, atol=1e-4 * np.abs(dv_ref).max())
        np.testing.assert_allclose(to_np(result.particle_qd), to_np(ref_out.particle_qd), rtol=0,
                                   atol=1e-4 * np.abs(dv_ref).max())
        np.testing.assert_allclose(to_np(result.particle_q), to_np(ref_out.particle_q), rtol=0, atol=1e-7)
        np.testing.assert_array_equal(to_np(result.particle_q)[fixed], to_np(model.particle_q)[fixed])
        np.testing.assert_array_equal(to_np(result.particle_qd)[fixed], 0.0)


def test_operator_preconditioner_diagonal_and_rhs_affinity():
    model, fixed, rng = mixed_model(seed=6)
    solver = solver_for(model, fixed)
    current = perturbed_state(model, rng)
    solver.refresh_tangent(current.particle_q)
    prepared = solver.prepare_step(current, None, None, DT)
    P = model.particle_count
    A = solver.A_bsr.dense().astype(np.float64)
    free = np.ones(3 * P, bool)
    for f in fixed:
        free[3 * f:3 * f + 3] = False
    PAP = A * np.outer(free, free) + np.diag((~free).astype(np.float64))
    vec = tensor(rng.normal(size=(P, 3)))
    out = torch.empty_like(vec)
    prepared.apply_operator(vec, out)
    want = (PAP @ to_np(vec).ravel()).reshape(P, 3)
    np.testing.assert_allclose(to_np(out), want, rtol=0, atol=2e-6 * np.abs(want).max())
    diag = to_np(prepared.diagonal_blocks)
    for i in range(P):
        np.testing.assert_allclose(diag[i], PAP[3 * i:3 * i + 3, 3 * i:3 * i + 3], rtol=1e-6, atol=1e-9)
    prepared.apply_preconditioner(vec, out)
    minv = to_np(solver._pc_inv_diag)
    np.testing.assert_allclose(to_np(out), np.einsum("nij,nj->ni", minv, to_np(vec)), rtol=1e-6, atol=1e-9)
    base = to_np(prepared.base_rhs)
    shifted = to_np(prepared.rhs(vec))
    expect = base + DT * to_np(vec) * free.reshape(P, 3)
    np.testing.assert_allclose(shifted, expect, rtol=2e-6, atol=1e-9)
    result = model.state()
    prepared.reconstruct(vec, result)  # no solve: pure kinematics from the prepared state
    q0, v0 = to_np(prepared._q), to_np(prepared._v)
    v_exp = v0 + to_np(vec)
    q_exp = q0 + DT * v_exp
    v_exp[fixed] = 0.0
    q_exp[fixed] = to_np(model.particle_q)[fixed]
    np.testing.assert_allclose(to_np(result.particle_qd), v_exp, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(to_np(result.particle_q), q_exp, rtol=1e-6, atol=1e-7)


def test_preparation_reuses_storage():
    model, fixed, rng = mixed_model(seed=7)
    solver = solver_for(model, fixed)
    current = perturbed_state(model, rng)
    solver.refresh_tangent(current.particle_q)
    prepared = solver.prepare_step(current, None, None, DT)
    pointers = (prepared.base_rhs.data_ptr(), prepared.velocity_increment.data_ptr(),
                prepared.diagonal_blocks.data_ptr())
    first = to_np(prepared.base_rhs).copy()
    current.particle_qd.mul_(2.0)
    again = solver.prepare_step(current, None, None, DT)
    assert again is prepared
    assert pointers == (again.base_rhs.data_ptr(), again.velocity_increment.data_ptr(),
                        again.diagonal_blocks.data_ptr())
    assert not np.array_equal(first, to_np(again.base_rhs))  # a new state re-evaluates the forces


def test_changed_timestep_requires_refresh_and_invalidates():
    model, fixed, rng = mixed_model(seed=8)
    solver = solver_for(model, fixed)
    current = perturbed_state(model, rng)
    solver.refresh_tangent(current.particle_q)
    prepared = solver.prepare_step(current, None, None, DT)
    smaller = DT / 2
    with pytest.raises(ValueError, match="assembled tangent"):
        solver.prepare_step(current, None, None, smaller)
    solver.refresh_tangent(current.particle_q, smaller)
    with pytest.raises(RuntimeError, match="changed"):
        prepared.rhs()
    prepared = solver.prepare_step(current, None, None, smaller)
    result = model.state()
    prepared.reconstruct(prepared.solve(prepared.base_rhs), result)
    ref_in, ref_out = copy_state(model, current), model.state()
    solver.step(ref_in, ref_out, None, None, smaller)
    np.testing.assert_allclose(to_np(result.particle_q), to_np(ref_out.particle_q), rtol=0, atol=1e-7)
    scale = np.abs(to_np(solver.velocity_increment)).max()
    np.testing.assert_allclose(to_np(result.particle_qd), to_np(ref_out.particle_qd), rtol=0, atol=1e-4 * scale)


def test_argument_checks_and_unprepared_workspace():
    model, fixed, rng = mixed_model(seed=9)
    solver = solver_for(model, fixed)
    current = perturbed_state(model, rng)
    with pytest.raises(RuntimeError, match="Prepare FEM mechanics"):
        PreparedFEMStep(solver).rhs()
    prepared = solver.prepare_step(current, None, None, DT)
    vec = torch.zeros_like(current.particle_q)
    with pytest.raises(ValueError, match="alias"):
        prepared.rhs(vec, vec)
    with pytest.raises(ValueError, match="distinct"):
        prepared.apply_operator(vec, vec)
    with pytest.raises(ValueError, match="distinct"):
        prepared.apply_preconditioner(vec, vec)
    with pytest.raises(ValueError, match="particle-sized"):
        prepared.rhs(torch.zeros(3, 3, device=DEVICE))
    bad = model.state()
    bad.particle_q = prepared._q
    with pytest.raises(ValueError, match="overwrite"):
        prepared.reconstruct(vec, bad)


def test_prepared_sequence_replays_in_a_cuda_graph():
    model, fixed, rng = mixed_model(seed=10)
    solver = solver_for(model, fixed, linear_solver_tolerance=1.0e-2, linear_solver_maxiter=50)
    current = perturbed_state(model, rng)
    solver.refresh_tangent(current.particle_q)
    prepared = solver.prepare_step(current, None, None, DT)
    load = torch.zeros_like(current.particle_q)
    result = model.state()
    guess = prepared.velocity_increment.clone()

    def trial():
        prepared.reconstruct(prepared.solve(prepared.rhs(load)), result)

    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        trial()  # warm-up outside capture
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            trial()
    for k in range(2):
        load.copy_(tensor(rng.normal(0, 0.3, tuple(load.shape))))
        prepared.velocity_increment.copy_(guess)
        graph.replay()
        torch.cuda.synchronize()
        q_graph = to_np(result.particle_q).copy()
        prepared.velocity_increment.copy_(guess)
        trial()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(q_graph, to_np(result.particle_q))


@pytest.mark.parametrize("stage", [4, 8])
def test_bulk_staged_operator_equals_direct_loads(stage):
    """fem_apply_operator with the block planes staged through shared memory by bulk asynchronous
    copies (FEM_TUNE_OPERATOR_STAGE) gives the direct kernel's result bit for bit (same products in the
    same order): mixed elements with fixed supports, slices whose length is not a multiple of the
    chunk, and the 64-row tail of a Hex8 block."""
    import ctypes

    from newton_solver_fem_gb300 import _lib, scenes

    lib = _lib.load()
    cases = [mixed_model(seed=7)]
    sc = scenes.hex_block_64(n=9)  # 1,000 nodes: a last slice of 8 rows
    from gpu_helpers import scene_pair

    hex_model, _, _ = scene_pair(sc, with_oracle=False)
    cases.append((hex_model, None, np.random.default_rng(8)))
    for model, fixed, rng in cases:
        solver = solver_for(model, fixed)
        solver.refresh_tangent(perturbed_state(model, rng).particle_q)
        P = model.particle_count
        x = tensor(rng.normal(size=(P, 3)))
        direct, staged = torch.empty_like(x), torch.empty_like(x)
        stream = torch.cuda.current_stream().cuda_stream
        _lib.check(lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_OPERATOR_STAGE, 0))
        _lib.check(lib.fem_apply_operator(solver._handle, x.data_ptr(), direct.data_ptr(), stream))
        _lib.check(lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_OPERATOR_STAGE, stage))
        v = ctypes.c_int64()
        _lib.check(lib.fem_get_tuning(solver._handle, _lib.FEM_TUNE_OPERATOR_STAGE, ctypes.byref(v)))
        assert v.value == stage
        _lib.check(lib.fem_apply_operator(solver._handle, x.data_ptr(), staged.data_ptr(), stream))
        torch.cuda.synchronize()
        assert solver.stats()["status"] == 0
        assert torch.equal(direct, staged)
