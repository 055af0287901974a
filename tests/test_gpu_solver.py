"""GPU parity of the C-ABI solver path against the CPU oracle (``-m gpu``).

Each test calls the library through ``SolverFEM`` (ctypes -> libfemgb300.so)
and compares with ``oracle.fem_oracle`` on the same float32 inputs, or restates
a reference test (file:line in the docstring) with its tolerance.  Tolerances:
element forces and assembled blocks rtol 1e-5 of the largest entry (float32
kernels vs the float64 oracle); one substep with a fixed CG iteration count
1e-4 relative L2 (SolverFEM parity bar); tolerance-driven solves by their true
residual; trajectories 1e-3 of the bounding-box diagonal.
"""

import numpy as np
import pytest
import torch
from fixtures import DT, cube_arrays, one_tet
from gpu_helpers import DEVICE, make_pair, rel_l2, rounded, scene_pair, small_batch, tensor, to_np

from newton_solver_fem_gb300 import FEMBuilder, SolverFEM, _lib, scenes
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _cuda(cuda_device):
    yield


def cube_pair(kind="tet", density=100.0, gravity=(0.0, 0.0, 0.0), **kw):
    x, el, mass, mats = cube_arrays(kind, density)
    args = dict(radius=0.004, gravity=gravity, dt=DT, min_stretch=-1.0, linear_solver_maxiter=128)
    args.update(kw)
    if kind == "tet":
        return make_pair(x, mass, tets=el, tet_materials=mats, **args)
    return make_pair(x, mass, hexes=el, hex_materials=mats, **args)


def deformed(x):
    q = x.copy()
    q[:, 0] *= 1.08
    q[:, 1] += 0.04 * q[:, 2]
    return q


# ---------------------------------------------------------------- element kernels


@pytest.mark.parametrize("kind", ["tet", "hex"])
def test_elastic_forces_match_oracle(kind):
    model, solver, oracle = cube_pair(kind, min_stretch=0.05)
    q = rounded(deformed(oracle.rest))
    v = rounded(np.random.default_rng(3).normal(0, 0.05, q.shape))
    state = model.state()
    state.particle_q.copy_(tensor(q))
    state.particle_qd.copy_(tensor(v))
    f = to_np(solver.eval_tetrahedral_forces(model, None, state) + solver.eval_hexahedral_forces(model, None, state))
    ref = oracle.forces(q, v, terms=("tet", "hex"))
    want = ref["tet"] + ref["hex"]
    np.testing.assert_allclose(f, want, rtol=0, atol=1e-5 * np.abs(want).max())


def test_hex_forces_on_distorted_cells_under_non_affine_motion_match_oracle():
    """Hex8 forces (elastic and damping) on jittered rest cells under a random non-affine deformation
    with random velocities.  For affine motion of box-shaped cells the bilinear and trilinear parts of
    dx/dxi vanish; here every part of the shape-function gradient contributes (kernels.py:1481-1601)."""
    rng = np.random.default_rng(17)
    x, hexes, mats, mass = scenes.hex_block(4, 3, 3, 0.05, (0.0, 0.0, 0.3), 2e5, 0.35, 1000.0, k_damp=0.02)
    x = x + rng.uniform(-0.005, 0.005, x.shape)
    model, solver, oracle = make_pair(x, mass, hexes=hexes, hex_materials=mats, min_stretch=0.05)
    q = rounded(oracle.rest + rng.normal(0.0, 0.004, x.shape))
    v = rounded(rng.normal(0.0, 0.1, x.shape))
    dN = O.hex_shape_gradients(oracle.hex_inv_J0)
    F = np.einsum("hai,hgaj->hgij", q[oracle.hexes], dN).reshape(-1, 3, 3)
    assert not O.clamp_active(F, 0.05, 20.0).any()
    state = model.state()
    state.particle_q.copy_(tensor(q))
    state.particle_qd.copy_(tensor(v))
    f = to_np(solver.eval_hexahedral_forces(model, None, state))
    want = oracle.forces(q, v, terms=("hex",))["hex"]
    np.testing.assert_allclose(f, want, rtol=0, atol=1e-5 * np.abs(want).max())


def test_tet_clamp_engages_on_inverted_element():
    """An inverted tet gives a negative smallest stretch that the clamp lifts (kernels.py:421-444)."""
    x, tets, mass, mats = one_tet()
    model, solver, oracle = make_pair(x, mass, tets=tets, tet_materials=mats, gravity=(0, 0, 0))
    q = rounded(x)
    q[3, 2] = -0.05  # invert
    assert O.clamp_active(O._cols(*(q[1:] - q[0])) @ oracle.tet_poses.astype(float), 0.05, 20.0).all()
    state = model.state()
    state.particle_q.copy_(tensor(q))
    f = to_np(solver.eval_tetrahedral_forces(model, None, state))
    want = oracle.forces(q, np.zeros_like(q), terms=("tet",))["tet"]
    np.testing.assert_allclose(f, want, rtol=0, atol=2e-5 * np.abs(want).max())


def test_springs_ground_gravity_damping_match_oracle():
    sc = scenes.tet_jittered_48(n=4)
    model, solver, oracle = scene_pair(sc, linear_damping=0.5)
    rng = np.random.default_rng(5)
    q = rounded(sc.x + rng.normal(0, 1e-3, sc.x.shape) - (0, 0, 0.203))  # some nodes below the ground
    v = rounded(rng.normal(0, 0.1, sc.x.shape))
    state = model.state()
    state.particle_q.copy_(tensor(q))
    state.particle_qd.copy_(tensor(v))
    ref = oracle.forces(q, v)
    for name, fn in (("spring", lambda: solver.eval_spring_forces(model, state)),
                     ("ground", lambda: solver.eval_particle_ground_contact_forces(model, None, state)),
                     ("gravity", lambda: solver.eval_gravity_forces(model)),
                     ("damping", lambda: solver.eval_linear_damping_forces(model, state))):
        got = to_np(fn())
        want = ref[name]
        assert np.abs(want).max() > 0, name
        np.testing.assert_allclose(got, want, rtol=0, atol=2e-6 * np.abs(want).max(), err_msg=name)


# ---------------------------------------------------------------- assembly


@pytest.mark.parametrize("kind", ["tet", "hex"])
def test_assembled_matrix_pattern_and_values(kind):
    model, solver, oracle = cube_pair(kind, min_stretch=0.05)
    q = rounded(deformed(oracle.rest))
    solver.refresh_tangent(tensor(q))
    oracle.refresh_tangent(q)
    A = solver.A_bsr
    np.testing.assert_array_equal(A.offsets.cpu().numpy(), oracle.offsets)
    np.testing.assert_array_equal(A.columns.cpu().numpy(), oracle.columns)
    vals = to_np(A.values)
    np.testing.assert_allclose(vals, oracle.values, rtol=0, atol=1e-5 * np.abs(oracle.values).max())
    minv = to_np(solver._pc_inv_diag)
    np.testing.assert_allclose(minv, oracle.minv, rtol=2e-4, atol=1e-6 * np.abs(oracle.minv).max())
    dense = A.dense()
    np.testing.assert_allclose(dense, dense.T, atol=2e-8 * max(1.0, np.abs(dense).max()))


@pytest.mark.parametrize("dims,loose", [((3, 2, 3), 0), ((5, 3, 2), 3)])
def test_hex_tangent_tail_alignment_clamp_and_negative_lambda(dims, loose):
    """Hex8 tangent blocks against the oracle where the kernel's special cases engage.

    * The hex count (18, 30) is not a multiple of the 16 hexes a CTA takes.
    * The first hex triplet sits at P (64 or 75 nodes with 3 loose particles): the last block plane is
      bulk-copied when that offset is a multiple of 4 floats, else stored by threads.
    * One node is pushed through its cell, so the stretch clamp engages (kernels.py:421-444).
    * Half of the hexes carry a negative lambda, and one hex a negative mu; this covers the signed
      path of the per-point factors.

    The element matrix is checked to be exactly symmetric, as the tiled kernel writes it."""
    nx, ny, nz = dims
    x, hexes, mats, mass = scenes.hex_block(nx, ny, nz, 0.1, (0.0, 0.0, 0.0), 2e4, 0.3, 1000.0)
    x = np.concatenate([x, 5.0 + np.arange(3 * loose, dtype=float).reshape(loose, 3)])
    mass = np.concatenate([mass, np.full(loose, 0.01)])
    mats = mats.copy()
    mats[::2, 1] *= -0.5
    mats[1, 0] *= -1.0
    model, solver, oracle = make_pair(x, mass, hexes=hexes, hex_materials=mats, min_stretch=0.05, max_stretch=20.0)
    q = rounded(deformed(oracle.rest))
    corner = hexes[len(hexes) // 2, 6]
    q[corner] = q[hexes[len(hexes) // 2, 0]] - 0.02
    dN = O.hex_shape_gradients(oracle.hex_inv_J0)
    F = np.einsum("hai,hgaj->hgij", q[oracle.hexes], dN).reshape(-1, 3, 3)
    assert O.clamp_active(F, 0.05, 20.0).any()
    solver.refresh_tangent(tensor(q))
    oracle.refresh_tangent(q)
    np.testing.assert_array_equal(solver.A_bsr.columns.cpu().numpy(), oracle.columns)
    vals = to_np(solver.A_bsr.values)
    np.testing.assert_allclose(vals, oracle.values, rtol=0, atol=1e-5 * np.abs(oracle.values).max())
    dense = solver.A_bsr.dense()
    assert np.array_equal(dense, dense.T)


def test_assembly_is_bitwise_deterministic():
    sc = scenes.hex_block_64(n=6)
    model, solver, _ = scene_pair(sc)
    q = model.particle_q + 1e-3 * torch.randn_like(model.particle_q)
    runs = []
    for _ in range(3):
        solver.refresh_tangent(q.clone())
        runs.append(solver.A_bsr.values.cpu().numpy().copy())
    for r in runs[1:]:
        assert np.array_equal(r, runs[0])


def test_triplet_layout_matches_reference_order():
    """bsr_values holds the reference's triplet layout [P | 2S | 16T] (solver.py:312-321)."""
    sc = scenes.tet_jittered_48(n=2)
    model, solver, oracle = scene_pair(sc)
    rows, cols, vals = (t.cpu().numpy() for t in solver._triplets())
    orow, ocol, oval = oracle.triplets(oracle.rest, oracle.dt)
    np.testing.assert_array_equal(rows, orow)
    np.testing.assert_array_equal(cols, ocol)
    np.testing.assert_allclose(vals, oval, rtol=0, atol=1e-5 * np.abs(oval).max())


# ---------------------------------------------------------------- solve


def test_fixed_iteration_substep_matches_oracle_cantilever():
    """One substep, K CG iterations (tolerance ~0): dv within 1e-4 relative L2 of the oracle."""
    sc = scenes.tet_cantilever()
    for K in (5, 20):
        model, solver, oracle = scene_pair(sc, linear_solver_maxiter=K, linear_solver_tolerance=1e-30)
        s0, s1 = model.state(), model.state()
        solver.step(s0, s1, None, None, sc.dt)
        _, v_ref, _ = oracle.step(oracle.rest, np.zeros_like(oracle.rest), sc.dt, fixed_iterations=K)
        assert solver.stats()["max_iterations"] == K
        assert rel_l2(to_np(solver.velocity_increment), oracle.dv) < 1e-4
        assert rel_l2(to_np(s1.particle_qd), v_ref) < 1e-4


def test_fixed_iteration_substep_matches_oracle_hex_with_ground_and_velocity():
    sc = scenes.hex_block_64(n=5)
    model, solver, oracle = scene_pair(sc, linear_solver_maxiter=15, linear_solver_tolerance=1e-30)
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, sc.dt)
    _, v_ref, rhs = oracle.step(rounded(sc.x), rounded(sc.velocity), sc.dt, fixed_iterations=15)
    assert rel_l2(to_np(solver.velocity_increment), oracle.dv) < 1e-4
    assert rel_l2(to_np(s0.particle_f), rhs) < 1e-5


def test_step_matches_dense_solve_and_preserves_inputs():
    """tests/test_solver.py:232-262 on the fast path at a tight tolerance (rtol 3e-4, atol 3e-6)."""
    model, solver, oracle = cube_pair("tet", linear_solver_tolerance=1e-7)
    s0, s1 = model.state(), model.state()
    q = to_np(s0.particle_q)
    q[-1, 2] -= 0.001
    velocity = rounded(np.random.default_rng(2).normal(0, 0.03, q.shape))
    force = np.zeros_like(q)
    force[-1] = (0.1, 0.05, -0.2)
    s0.particle_q.copy_(tensor(q))
    s0.particle_qd.copy_(tensor(velocity))
    ext = tensor(force)
    A = solver.A_bsr.dense()
    elastic = to_np(solver.eval_tetrahedral_forces(model, None, s0))
    mass = np.repeat(to_np(model.particle_mass), 3)
    rhs = DT * (force + elastic).ravel() - A @ velocity.ravel() + mass * velocity.ravel()
    inc = np.linalg.solve(A, rhs).reshape(q.shape)
    solver.step(s0, s1, None, None, DT, external_forces=ext)
    np.testing.assert_allclose(to_np(s1.particle_qd), velocity + inc, rtol=3e-4, atol=3e-6)
    np.testing.assert_allclose(to_np(s1.particle_q), q + DT * (velocity + inc), rtol=1e-6, atol=1e-7)
    np.testing.assert_array_equal(to_np(s0.particle_q), rounded(q))
    np.testing.assert_array_equal(to_np(ext), rounded(force))


@pytest.mark.parametrize("tol", [1e-2, 1e-5])
def test_true_residual_meets_tolerance_fp64(tol):
    """||A dv - b|| / ||b|| <= tol (x1.01) re-checked in float64 (tests/test_solver.py:281-316, 535-538)."""
    model, solver, _ = cube_pair("tet", linear_solver_tolerance=tol)
    ext = tensor(np.random.default_rng(13).normal(0, 0.03, (model.particle_count, 3)))
    s0, s1 = model.state(), model.state()
    solver.velocity_increment.zero_()
    solver.step(s0, s1, None, None, DT, external_forces=ext)
    A = solver.A_bsr.dense()
    rhs = to_np(s0.particle_f).ravel()
    res = np.linalg.norm(A @ to_np(solver.velocity_increment).ravel() - rhs) / np.linalg.norm(rhs)
    assert res < tol * 1.01 + 1e-6


def test_tolerance_change_changes_iterations():
    model, solver, _ = cube_pair("tet")
    ext = tensor(np.random.default_rng(13).normal(0, 0.03, (model.particle_count, 3)))
    its = []
    for tol in (1e-2, 1e-5, 1e-2):
        solver.linear_solver_tolerance = tol
        solver.velocity_increment.zero_()
        s0, s1 = model.state(), model.state()
        solver.step(s0, s1, None, None, DT, external_forces=ext)
        its.append(solver.last_cg_iters)
    assert its[1] > its[0] and its[0] == its[2]
    with pytest.raises(ValueError):
        solver.linear_solver_tolerance = 0.0


@pytest.mark.parametrize("density", [0.1, 1000.0])
def test_freefall_across_mass_scales(density):
    """tests/test_solver.py:440-450 (checked-solve tolerance)."""
    model, solver, _ = cube_pair("tet", density=density, linear_solver_tolerance=1e-8)
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, DT)
    np.testing.assert_allclose(to_np(s1.particle_q), to_np(s0.particle_q), atol=2e-7)
    model.set_gravity((0, 0, -9.81))
    solver.step(s0, s1, None, None, DT)
    np.testing.assert_allclose(to_np(s1.particle_qd)[:, 2], -DT * 9.81, atol=2e-5)


@pytest.mark.parametrize("mass", [1e-25, 1e-18, 1e-14, 1.0])
def test_tiny_mass_falls_and_zero_rhs_clears_warm_start(mass):
    """tests/test_reference_block_preconditioner.py:71-91."""
    dt = 1 / 240
    b = FEMBuilder(gravity=(0.0, 0.0, -9.81))
    b.add_particle((0, 0, 1), (0, 0, 0), mass=mass)
    model = b.finalize(DEVICE)
    solver = SolverFEM(model, dt=dt, solver_type="cg", preconditioner_type="block_diag", linear_solver_maxiter=8,
                       self_contact_ke=0.0)
    cur, nxt = model.state(), model.state()
    ptr = solver.velocity_increment.data_ptr()
    for step in range(1, 4):
        solver.step(cur, nxt, model.control(), None, dt)
        np.testing.assert_allclose(to_np(nxt.particle_qd)[0], (0, 0, -step * 9.81 * dt), atol=1e-7)
        np.testing.assert_allclose(to_np(solver.velocity_increment)[0], (0, 0, -9.81 * dt), atol=1e-7)
        np.testing.assert_allclose(to_np(cur.particle_f)[0], (0, 0, -mass * 9.81 * dt), rtol=3e-7, atol=0)
        assert solver.velocity_increment.data_ptr() == ptr
        cur, nxt = nxt, cur
    model.set_gravity((0, 0, 0))
    solver.step(cur, nxt, model.control(), None, dt)
    np.testing.assert_allclose(to_np(nxt.particle_qd), to_np(cur.particle_qd), atol=1e-7)
    np.testing.assert_array_equal(to_np(solver.velocity_increment), np.zeros((1, 3)))


def test_hex_box_one_step_known_answer():
    """tests/test_reference_builder.py:35-54: dv_z = -0.00981."""
    b = FEMBuilder(gravity=(0.0, 0.0, -9.81))
    nodes = np.asarray([(0, 0, 0), (2, 0, 0), (2, 3, 0), (0, 3, 0), (0, 0, 4), (2, 0, 4), (2, 3, 4), (0, 3, 4)], float)
    b.add_particles(nodes, np.zeros_like(nodes), [3.0] * 8)
    b.add_soft_hex_mesh(np.arange(8).reshape(1, 8), k_mu=10.0, k_lambda=20.0, k_damp=0.0)
    model = b.finalize(DEVICE)
    np.testing.assert_allclose(to_np(model.fem.hex_det_J0_w), 3.0)
    solver = SolverFEM(model, dt=0.001, preconditioner_type="block_diag", solver_type="cg", self_contact_ke=0.0)
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, 0.001)
    np.testing.assert_allclose(to_np(s1.particle_qd)[:, 2], -0.00981, atol=1e-7)


def test_dirichlet_matches_reduced_system():
    """tests/test_fixed_particles.py:50-79 (rtol 3e-4, atol 2e-6), including refresh_tangent."""
    x, tets, mass, mats = one_tet()
    model, solver, _ = make_pair(x, mass, tets=tets, tet_materials=mats, gravity=(0, 0, 0), fixed=[0, 1], dt=DT,
                                 linear_solver_maxiter=64, linear_solver_tolerance=1e-7)
    cur, nxt = model.state(), model.state()
    rest = to_np(model.particle_q)
    q = rest.copy()
    q[2] += (0.002, 0.001, -0.001)
    velocity = np.array(((0, 0, 0), (0, 0, 0), (0.02, -0.03, 0.01), (-0.01, 0.01, 0.02)), np.float32)
    external = np.array(((20, 30, 40), (10, -30, 60), (0.02, 0.04, 0.03), (-0.01, 0.03, 0.02)), np.float32)
    forces = tensor(external)
    cur.particle_q.copy_(tensor(q))
    cur.particle_qd.copy_(tensor(velocity))
    for refresh in (False, True, True):
        if refresh:
            solver.refresh_tangent(cur.particle_q)
        A = solver.A_bsr.dense()
        elastic = to_np(solver.eval_tetrahedral_forces(model, None, cur))
        m = np.repeat(to_np(model.particle_mass), 3)
        rhs = DT * (elastic + external).ravel() - (A - np.diag(m)) @ velocity.ravel().astype(np.float64)
        expected = np.zeros(12)
        expected[6:] = np.linalg.solve(A[6:, 6:], rhs[6:])
        solver.step(cur, nxt, None, None, DT, external_forces=forces)
        np.testing.assert_allclose(to_np(solver.velocity_increment).ravel(), expected, rtol=3e-4, atol=2e-6)
        np.testing.assert_array_equal(to_np(nxt.particle_q)[:2], rest[:2])
        np.testing.assert_array_equal(to_np(nxt.particle_qd)[:2], np.zeros((2, 3)))
        np.testing.assert_array_equal(solver.A_bsr.dense(), A)
        cur, nxt = nxt, cur
        velocity = to_np(cur.particle_qd).astype(np.float32)


def test_boundary_restored_after_external_state_changes():
    """tests/test_fixed_particles.py:81-90."""
    x, tets, mass, mats = one_tet()
    model, solver, _ = make_pair(x, mass, tets=tets, tet_materials=mats, gravity=(0, 0, 0), fixed=[0, 1, 2, 3], dt=DT)
    cur, nxt = model.state(), model.state()
    cur.particle_q.fill_(0.5)
    cur.particle_qd.fill_(100.0)
    solver.step(cur, nxt, None, None, DT)
    np.testing.assert_array_equal(to_np(nxt.particle_q), to_np(model.particle_q))
    np.testing.assert_array_equal(to_np(nxt.particle_qd), np.zeros((4, 3)))
    np.testing.assert_array_equal(to_np(solver.velocity_increment), np.zeros((4, 3)))


def test_invalid_arguments_rejected():
    """tests/test_fixed_particles.py:112-121 and tests/test_solver.py:241-262 validation."""
    x, tets, mass, mats = one_tet()
    model, _, _ = make_pair(x, mass, tets=tets, tet_materials=mats, gravity=(0, 0, 0))
    for indices in ((-1,), (4,), (1.0,), ((1, 2),)):
        with pytest.raises(ValueError):
            SolverFEM(model, fixed_particle_indices=indices, solver_type="cg", self_contact_ke=0)
    for tol in (0.0, -1e-5, float("nan"), float("inf")):
        with pytest.raises(ValueError, match="finite and positive"):
            SolverFEM(model, solver_type="cg", linear_solver_tolerance=tol)
    solver = SolverFEM(model, solver_type="cg", preconditioner_type="block_diag", self_contact_ke=0)
    s0, s1 = model.state(), model.state()
    with pytest.raises(ValueError):
        solver.step(s0, s1, None, None, DT, external_forces=torch.zeros(3, 3, device=DEVICE))


def test_trajectory_cantilever_60_frames_within_bbox_tolerance():
    """60 frames x 10 substeps of the Tet4 cantilever at tol 1e-2 stay within 1e-3 bbox diagonal of the oracle."""
    sc = scenes.tet_cantilever()
    model, solver, oracle = scene_pair(sc)
    cur, nxt = model.state(), model.state()
    q, v = oracle.rest.copy(), np.zeros_like(oracle.rest)
    diag = np.linalg.norm(np.ptp(sc.x, axis=0))
    worst = 0.0
    for frame in range(60):
        solver.refresh_tangent(cur.particle_q)
        q = oracle.refresh_tangent(q)
        for _ in range(sc.substeps):
            solver.step(cur, nxt, None, None, sc.dt)
            cur, nxt = nxt, cur
            q, v, _ = oracle.step(q, v, sc.dt)
        worst = max(worst, np.abs(to_np(cur.particle_q) - q).max() / diag)
    assert worst < 1e-3, worst
    assert np.isfinite(to_np(cur.particle_q)).all()


# ---------------------------------------------------------------- graphs, batching, failure detection


def test_captured_graph_matches_eager_with_live_inputs():
    """Capture refresh_tangent + substeps; replay with changed external forces and gravity equals eager steps."""
    sc = scenes.tet_cantilever()
    model_a, solver_a, _ = scene_pair(sc)
    model_b, solver_b, _ = scene_pair(sc)
    ext_a = torch.zeros((model_a.particle_count, 3), device=DEVICE)
    ext_b = torch.zeros_like(ext_a)
    a0, a1 = model_a.state(), model_a.state()
    b0, b1 = model_b.state(), model_b.state()
    # warm up (first refresh, solver setup) outside capture
    solver_a.refresh_tangent(a0.particle_q)
    solver_a.step(a0, a1, None, None, sc.dt, external_forces=ext_a)
    solver_b.refresh_tangent(b0.particle_q)
    solver_b.step(b0, b1, None, None, sc.dt, external_forces=ext_b)
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            solver_a.refresh_tangent(a0.particle_q)
            solver_a.step(a0, a1, None, None, sc.dt, external_forces=ext_a)
            solver_a.step(a1, a0, None, None, sc.dt, external_forces=ext_a)
    for scale, g in ((1.0, -9.81), (-2.0, -4.0), (0.0, 0.0)):
        force = np.zeros((model_a.particle_count, 3), np.float32)
        force[-1] = (0.2 * scale, 0.0, -0.1 * scale)
        ext_a.copy_(tensor(force))
        ext_b.copy_(tensor(force))
        model_a.set_gravity((0, 0, g))
        model_b.set_gravity((0, 0, g))
        graph.replay()
        solver_b.refresh_tangent(b0.particle_q)
        solver_b.step(b0, b1, None, None, sc.dt, external_forces=ext_b)
        solver_b.step(b1, b0, None, None, sc.dt, external_forces=ext_b)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(to_np(a0.particle_q), to_np(b0.particle_q))
        np.testing.assert_array_equal(to_np(a0.particle_qd), to_np(b0.particle_qd))


def test_batched_scenes_match_individual_solves():
    """Scenes packed in one handle (per-scene CG scalars and convergence) equal each scene solved alone."""
    check_batch_against_solo_solves(small_batch())


def test_spread_batch_matches_individual_solves():
    """24 scenes of up to 10^3 cells: each scene's slices are dealt to several CTAs in interleaved
    runs, and its reductions sum segments from many CTAs; the result still equals each scene alone."""
    check_batch_against_solo_solves(scenes.batched_scenes(count=24, seed=5, dims=(3, 10)))


def check_batch_against_solo_solves(sc):
    model, solver, _ = scene_pair(sc)
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, sc.dt)
    stats = solver.stats()
    dv = to_np(solver.velocity_increment)
    offs = sc.scene_offsets
    assert len(stats["scene_iterations"]) == len(offs) - 1
    for s in range(len(offs) - 1):
        lo, hi = offs[s], offs[s + 1]
        x = sc.x[lo:hi]
        tet_sel = np.all((sc.tets >= lo) & (sc.tets < hi), axis=1)
        hex_sel = np.all((sc.hexes >= lo) & (sc.hexes < hi), axis=1)
        fixed = sc.fixed[(sc.fixed >= lo) & (sc.fixed < hi)] - lo
        kw = dict(fixed=fixed, dt=sc.dt, linear_solver_maxiter=sc.maxiter, linear_solver_tolerance=sc.tolerance)
        if tet_sel.any():
            kw.update(tets=sc.tets[tet_sel] - lo, tet_materials=sc.tet_materials[tet_sel])
        if hex_sel.any():
            kw.update(hexes=sc.hexes[hex_sel] - lo, hex_materials=sc.hex_materials[hex_sel])
        m1, s_one, _ = make_pair(x, sc.mass[lo:hi], **kw)
        a0, a1 = m1.state(), m1.state()
        s_one.step(a0, a1, None, None, sc.dt)
        assert s_one.stats()["max_iterations"] == stats["scene_iterations"][s]
        np.testing.assert_allclose(dv[lo:hi], to_np(s_one.velocity_increment), rtol=1e-5,
                                   atol=1e-6 * np.abs(dv[lo:hi]).max())


def test_batched_scenes_match_oracle_fixed_iterations():
    sc = small_batch(count=4, seed=3)
    model, solver, oracle = scene_pair(sc, linear_solver_maxiter=10, linear_solver_tolerance=1e-30)
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, sc.dt)
    oracle.step(oracle.rest, np.zeros_like(oracle.rest), sc.dt, fixed_iterations=10)
    offs = sc.scene_offsets
    dv = to_np(solver.velocity_increment)
    for s in range(len(offs) - 1):
        sl = slice(offs[s], offs[s + 1])
        assert rel_l2(dv[sl], oracle.dv[sl]) < 1e-4


def test_single_reduction_cg_matches_oracle_fixed_iterations_on_a_batch():
    """The single-reduction (Chronopoulos-Gear) recurrence is CG: at a fixed iteration count each scene of
    a batch (fixed faces, spread over CTAs) matches the oracle's standard PCG."""
    sc = scenes.batched_scenes(count=24, seed=5, dims=(3, 10))
    model, solver, oracle = scene_pair(sc, linear_solver_maxiter=10, linear_solver_tolerance=1e-30)
    _lib.check(_lib.load().fem_set_tuning(solver._handle, _lib.FEM_TUNE_CG_VARIANT, 1))
    rng = np.random.default_rng(8)
    q = rounded(sc.x + rng.normal(0, 0.001, sc.x.shape))
    q[sc.fixed] = rounded(sc.x[sc.fixed])
    v = rounded(rng.normal(0, 0.05, sc.x.shape))
    v[sc.fixed] = 0.0
    s0, s1 = model.state(), model.state()
    s0.particle_q.copy_(tensor(q))
    s0.particle_qd.copy_(tensor(v))
    solver.refresh_tangent(s0.particle_q)
    solver.step(s0, s1, None, None, sc.dt)
    stats = solver.stats()
    assert stats["scene_iterations"] == [10] * (len(sc.scene_offsets) - 1)
    oracle.refresh_tangent(q)
    oracle.step(q, v, sc.dt, fixed_iterations=10)
    dv = to_np(solver.velocity_increment)
    offs = sc.scene_offsets
    for s in range(len(offs) - 1):
        sl = slice(offs[s], offs[s + 1])
        assert rel_l2(dv[sl], oracle.dv[sl]) < 1e-4, s


def test_barrier_wait_limit_reports_timeout_and_recovers():
    """A bounded grid-barrier wait that runs out returns a status, not a hang or fault; the context stays usable."""
    sc = scenes.hex_block_64(n=24)  # many CTAs in the cooperative grid
    model, solver, _ = scene_pair(sc, with_oracle=False)
    s0, s1 = model.state(), model.state()
    lib = _lib.load()
    _lib.check(lib.fem_set_wait_limit(solver._handle, 0))
    solver.step(s0, s1, None, None, sc.dt)
    with pytest.raises(_lib.FemError) as err:
        solver.stats()
    assert err.value.code == _lib.FEM_ERR_TIMEOUT
    _lib.check(lib.fem_set_wait_limit(solver._handle, 2_000_000_000))
    solver.reset()
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, sc.dt)
    assert solver.stats()["status"] == 0
    assert np.isfinite(to_np(s1.particle_q)).all()


def test_large_hex_block_true_residual_property():
    """Full-size Hex8 64^3 block: one substep's true relative residual <= tol, re-checked in float64."""
    sp = pytest.importorskip("scipy.sparse")
    sc = scenes.hex_block_64()
    model, solver, _ = scene_pair(sc, with_oracle=False)
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, sc.dt)
    st = solver.stats()
    A = solver.A_bsr
    P = model.particle_count
    M = sp.bsr_matrix((A.values.cpu().numpy().astype(np.float64), A.columns.cpu().numpy(),
                       A.offsets.cpu().numpy()), shape=(3 * P, 3 * P))
    rhs = to_np(s0.particle_f).ravel()
    res = np.linalg.norm(M @ to_np(solver.velocity_increment).ravel() - rhs) / np.linalg.norm(rhs)
    assert st["unconverged_scenes"] == 0 and st["max_iterations"] <= 50, st
    assert res < 1e-2 * 1.01, res
    assert np.isfinite(to_np(s1.particle_q)).all()


def test_full_size_jittered_tet_block_with_springs_and_ground():
    """Full-size jittered Tet4 48^3 block (663,552 tets, 795,024 edge springs, ground): 3 frames of
    10 substeps stay finite, every solve converges within its iteration cap, and the last substep's
    true relative residual is re-checked in float64."""
    sp = pytest.importorskip("scipy.sparse")
    sc = scenes.tet_jittered_48()
    model, solver, _ = scene_pair(sc, with_oracle=False)
    a, b = model.state(), model.state()
    for frame in range(3):
        solver.refresh_tangent(a.particle_q)
        for k in range(sc.substeps):
            solver.step(a, b, None, None, sc.dt)
            st = solver.stats()
            assert st["max_iterations"] <= sc.maxiter and st["unconverged_scenes"] == 0, st
            a, b = b, a
    A = solver.A_bsr
    P = model.particle_count
    assert A.columns.numel() == 1_707_697  # stored 3x3 blocks of the jittered Tet4 48^3 block with its edge springs
    M = sp.bsr_matrix((A.values.cpu().numpy().astype(np.float64), A.columns.cpu().numpy(),
                       A.offsets.cpu().numpy()), shape=(3 * P, 3 * P))
    rhs = to_np(b.particle_f).ravel()
    res = np.linalg.norm(M @ to_np(solver.velocity_increment).ravel() - rhs) / np.linalg.norm(rhs)
    assert st["unconverged_scenes"] == 0, st
    assert res < sc.tolerance * 1.01, res
    q = to_np(a.particle_q)
    assert np.isfinite(q).all()
    assert q[:, 2].min() > -0.01  # the ground holds the block (penetration below 1 cm)
