"""Adjoint (differentiable) path on the GPU vs float64 central differences of the oracle (``-m gpu``).

The matrix is frozen during differentiation (the reference's contract,
differentiation.py:1-8), so the oracle's finite differences perturb forces,
states and controls with A held at its nominal assembly.  Tolerance 1e-3
relative (float32 adjoint vs float64 differences), the differentiable-beam bar.
"""

import time
from pathlib import Path

import numpy as np
import pytest
import torch
from gpu_helpers import DEVICE, make_pair, rounded, scene_pair, tensor, to_np

from newton_solver_fem_gb300 import FEMBuilder, SolverFEM, _lib, scenes
from newton_solver_fem_gb300.adjoint import DifferentiableSolver, checkpointed_gradient
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _cuda(cuda_device):
    yield


def small_beam(nx=4, fixed=True, seed=0):
    x, tets, mats, mass = scenes.tet_block(nx, 1, 1, 0.05, (0, 0, 0), 1.0e5, 0.45, 1000.0)
    rng = np.random.default_rng(seed)
    scale = rng.uniform(0.8, 1.2, size=len(tets)).astype(np.float32)
    fx = np.nonzero(np.isclose(x[:, 0], 0.0))[0].astype(np.int32) if fixed else None
    return x, tets, mats, mass, scale, fx


def _vjp(solver, q, v, g, act=None):
    lib = _lib.load()
    qb = torch.zeros_like(q)
    vb = torch.zeros_like(v)
    T = solver.model.tet_count
    ab = torch.zeros(T, device=DEVICE) if T else None
    sb = torch.zeros(T, device=DEVICE) if T else None
    _lib.check(lib.fem_force_vjp(solver._handle, q.data_ptr(), v.data_ptr(), None if act is None else act.data_ptr(),
                                 solver.model.gravity.data_ptr(), g.data_ptr(), qb.data_ptr(), vb.data_ptr(),
                                 None if ab is None else ab.data_ptr(), None if sb is None else sb.data_ptr(),
                                 torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return to_np(qb), to_np(vb), None if ab is None else to_np(ab), None if sb is None else to_np(sb)


def _assert_clamp_inactive(oracle, q):
    """The VJP differentiates the stretch clamp as the identity; check the state leaves it inactive."""
    lo, hi = oracle.min_stretch, oracle.max_stretch
    if len(oracle.tets):
        t = oracle.tets
        Ds = np.stack([q[t[:, k]] - q[t[:, 0]] for k in (1, 2, 3)], axis=-1)
        assert not O.clamp_active(Ds @ oracle.tet_poses, lo, hi).any()
    if len(oracle.hexes):
        dN = O.hex_shape_gradients(oracle.hex_inv_J0)
        F = np.einsum("hai,hgaj->hgij", q[oracle.hexes], dN).reshape(-1, 3, 3)
        assert not O.clamp_active(F, lo, hi).any()


def _total_force(oracle, q, v, activation=None):
    return sum(oracle.forces(q, v, activation=activation).values())


@pytest.mark.parametrize("case", ["tet_act_scale", "hex", "springs_ground_damping"])
def test_force_vjp_directional_derivatives(case):
    rng = np.random.default_rng(11)
    act = None
    if case == "tet_act_scale":
        x, tets, mats, mass, scale, _ = small_beam(fixed=False)
        model, solver, oracle = make_pair(x, mass, tets=tets, tet_materials=mats, gravity=(0, 0, -9.81),
                                          enable_tet_activations=True)
        diff = DifferentiableSolver(solver)
        diff.set_mu_scale(tensor(scale))
        oracle.mu_scale = scale.astype(np.float64)
        act_np = rounded(rng.uniform(-0.2, 0.2, len(tets)))
        act = tensor(act_np)
    elif case == "hex":
        sc = scenes.hex_block_64(n=3)
        model, solver, oracle = scene_pair(sc)
        act_np = None
    else:
        sc = scenes.tet_jittered_48(n=3)
        model, solver, oracle = scene_pair(sc, linear_damping=0.7)
        act_np = None
    x = oracle.rest
    cell = 0.05 if case == "tet_act_scale" else 0.01
    q = rounded(x + rng.normal(0, 0.02 * cell, x.shape))
    if case == "springs_ground_damping":
        q = rounded(q - (0, 0, 0.2015))  # bottom layer 1.5 mm into the ground
    _assert_clamp_inactive(oracle, q)
    v = rounded(rng.normal(0, 0.05, x.shape))
    g = rounded(rng.normal(0, 1.0, x.shape))
    qb, vb, ab, sb = _vjp(solver, tensor(q), tensor(v), tensor(g), act)
    eps = 1e-6
    for k in range(3):
        dq = rng.normal(size=x.shape)
        dv = rng.normal(size=x.shape)
        fq = (_total_force(oracle, q + eps * dq, v, act_np) - _total_force(oracle, q - eps * dq, v, act_np)) / (2 * eps)
        fv = (_total_force(oracle, q, v + eps * dv, act_np) - _total_force(oracle, q, v - eps * dv, act_np)) / (2 * eps)
        want_q, want_v = float(np.sum(g * fq)), float(np.sum(g * fv))
        np.testing.assert_allclose(np.sum(qb * dq), want_q, rtol=1e-3, atol=1e-4 * (abs(want_q) + 1e-8))
        if abs(want_v) > 1e-10:
            np.testing.assert_allclose(np.sum(vb * dv), want_v, rtol=1e-3, atol=1e-6)
    if case == "tet_act_scale":
        da = rng.normal(size=len(act_np))
        fa = (_total_force(oracle, q, v, act_np + eps * da) - _total_force(oracle, q, v, act_np - eps * da)) / (2 * eps)
        np.testing.assert_allclose(np.sum(ab * da), np.sum(g * fa), rtol=1e-3)
        ds = rng.normal(size=len(scale))
        base = oracle.mu_scale.copy()
        oracle.mu_scale = base + eps * ds
        fp = _total_force(oracle, q, v, act_np)
        oracle.mu_scale = base - eps * ds
        fm = _total_force(oracle, q, v, act_np)
        oracle.mu_scale = base
        np.testing.assert_allclose(np.sum(sb * ds), np.sum(g * (fp - fm) / (2 * eps)), rtol=1e-3)


def _oracle_rollout(oracle, q, v, exts, dt, scale=None):
    if scale is not None:
        oracle.mu_scale = scale
    oracle.dv[:] = 0.0
    for ext in exts:
        oracle.dv[:] = 0.0
        q, v, _ = oracle.step(q, v, dt, external=ext)
    return q, v


def test_multistep_gradients_match_oracle_differences():
    """Gradients wrt q0, v0, external forces and the shear scale over 4 substeps (fixed end, gravity)."""
    x, tets, mats, mass, scale, fixed = small_beam()
    dt = 1.0 / 240.0
    model, solver, oracle = make_pair(x, mass, tets=tets, tet_materials=mats, gravity=(0, 0, -9.81), fixed=fixed,
                                      dt=dt, linear_solver_maxiter=200)
    oracle = O.OracleFEM(oracle.rest, oracle.mass, tets=tets, tet_poses=oracle.tet_poses, tet_materials=mats,
                         gravity=(0, 0, -9.81), fixed=fixed, dt=dt, maxiter=400, tolerance=1e-13,
                         mu_scale=scale.astype(np.float64))
    diff = DifferentiableSolver(solver, tolerance=1e-7, maxiter=200)
    s_t = tensor(scale).requires_grad_(True)
    diff.set_mu_scale(s_t)
    solver.refresh_tangent(model.particle_q.clone())  # A at the nominal scale, frozen from here on
    rng = np.random.default_rng(3)
    q0 = rounded(oracle.rest + rng.normal(0, 1e-3, x.shape))
    q0[fixed] = oracle.rest[fixed]
    v0 = rounded(rng.normal(0, 0.02, x.shape))
    v0[fixed] = 0.0
    exts = [rounded(rng.normal(0, 0.01, x.shape)) for _ in range(4)]
    w = rng.normal(size=x.shape)
    wv = rng.normal(size=x.shape)

    def loss_np(q, v):
        return float(np.sum(w * q) + 0.5 * np.sum(wv * v))

    qt = tensor(q0).requires_grad_(True)
    vt = tensor(v0).requires_grad_(True)
    et = [tensor(e).requires_grad_(True) for e in exts]
    q, v = qt, vt
    for k in range(4):
        q, v = diff.step(q, v, dt, external_forces=et[k], mu_scale=s_t)
    loss = (torch.tensor(w, device=DEVICE, dtype=torch.float32) * q).sum() + \
        0.5 * (torch.tensor(wv, device=DEVICE, dtype=torch.float32) * v).sum()
    loss.backward()
    grads = {"q0": to_np(qt.grad), "v0": to_np(vt.grad), "ext": sum(to_np(e.grad) for e in et) / 1.0,
             "scale": to_np(s_t.grad)}
    eps = {"q0": 1e-5, "v0": 1e-4, "ext": 1e-4, "scale": 1e-4}
    for name in ("q0", "v0", "ext", "scale"):
        d = rng.normal(size=scale.shape if name == "scale" else x.shape)
        if name in ("q0", "v0"):
            d[fixed] = 0.0
        vals = []
        for sgn in (1.0, -1.0):
            qq, vv, ee, ss = q0.copy(), v0.copy(), [e.copy() for e in exts], scale.astype(np.float64)
            if name == "q0":
                qq = qq + sgn * eps[name] * d
            elif name == "v0":
                vv = vv + sgn * eps[name] * d
            elif name == "ext":
                ee = [e + sgn * eps[name] * d for e in ee]
            else:
                ss = ss + sgn * eps[name] * d
            vals.append(loss_np(*_oracle_rollout(oracle, qq, vv, ee, dt, ss)))
        fd = (vals[0] - vals[1]) / (2 * eps[name])
        exact = float(np.sum(grads[name] * d))
        assert abs(exact - fd) <= 1e-3 * abs(fd) + 1e-7, (name, exact, fd)


def test_checkpointed_gradient_equals_full_tape():
    """Segment recomputation gives the same gradients as one recorded rollout (tests/test_bear_training.py:76-138)."""
    x, tets, mats, mass, scale, fixed = small_beam()
    dt = 1.0 / 240.0
    model, solver, _ = make_pair(x, mass, tets=tets, tet_materials=mats, gravity=(0, 0, -9.81), fixed=fixed, dt=dt,
                                 linear_solver_maxiter=200, with_oracle=False)
    diff = DifferentiableSolver(solver, tolerance=1e-7, maxiter=200)
    s_t = tensor(scale).requires_grad_(True)
    diff.set_mu_scale(s_t)
    solver.refresh_tangent(model.particle_q.clone())
    q0 = model.particle_q.clone()
    v0 = torch.zeros_like(q0)
    target = q0.mean(0) - torch.tensor([0.0, 0.0, 0.01], device=DEVICE)

    def step(q, v, k):
        return diff.step(q, v, dt, mu_scale=s_t)

    def loss_fn(q, v):
        return ((q.mean(0) - target) ** 2).sum()

    loss_c, _, vb_c, (gs_c,) = checkpointed_gradient(step, q0, v0, 12, 4, loss_fn, params=(s_t,))
    qt, vt = q0.clone(), v0.clone().requires_grad_(True)
    q, v = qt, vt
    for k in range(12):
        q, v = step(q, v, k)
    loss_f = loss_fn(q, v)
    gs_f, vb_f = torch.autograd.grad(loss_f, (s_t, vt))
    np.testing.assert_allclose(loss_c.item(), loss_f.item(), rtol=1e-6)
    np.testing.assert_allclose(to_np(gs_c), to_np(gs_f), rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(to_np(vb_c), to_np(vb_f), rtol=1e-5, atol=1e-12)


def test_external_force_derivative_is_half_dt():
    """A free 2 kg particle: d v_x / d f_ext = h/2 (tests/test_solver.py:452-464)."""
    b = FEMBuilder(gravity=(0.0, 0.0, 0.0))
    b.add_particle((0, 0, 1), (0, 0, 0), mass=2.0)
    model = b.finalize(DEVICE)
    dt = 0.002
    solver = SolverFEM(model, dt=dt, solver_type="cg", preconditioner_type="block_diag", self_contact_ke=0.0,
                       linear_solver_maxiter=128)
    diff = DifferentiableSolver(solver)
    ext = torch.zeros((1, 3), device=DEVICE, requires_grad=True)
    s = model.state()
    q, v = diff.step(s.particle_q, s.particle_qd, dt, external_forces=ext)
    v[:, 0].sum().backward()
    np.testing.assert_allclose(to_np(ext.grad), [[dt / 2, 0, 0]], atol=1e-8)


GOLDEN = Path(__file__).with_name("golden")


def beam_problem():
    """The differentiable beam (16x4x4 cubes, 1,536 tets) with its shear scales bound as a leaf tensor."""
    sc = scenes.tet_beam()
    model, solver, _ = make_pair(sc.x, sc.mass, tets=sc.tets, tet_materials=sc.tet_materials, fixed=sc.fixed,
                                 dt=sc.dt, linear_solver_maxiter=sc.maxiter, with_oracle=False)
    diff = DifferentiableSolver(solver, tolerance=1.0e-8, maxiter=sc.maxiter)
    s_t = tensor(sc.extra["mu_scale"]).requires_grad_(True)
    diff.set_mu_scale(s_t)
    solver.refresh_tangent(model.particle_q.clone())  # A at the nominal scales, frozen from here on
    tip = torch.as_tensor(sc.extra["tip_nodes"], device=DEVICE, dtype=torch.long)
    target = tensor(sc.extra["target"])

    def step(q, v, k):
        return diff.step(q, v, sc.dt, mu_scale=s_t)

    def loss_fn(q, v):
        return ((q[tip].mean(0) - target) ** 2).sum()

    return sc, model, s_t, step, loss_fn


def test_beam_checkpointed_gradient_matches_fp64_differences():
    """120 frames x 4 substeps, checkpoints every 10 frames, vs float64 central differences (eps 1e-3)."""
    fx = np.load(GOLDEN / "beam_fd.npz")
    sc, model, s_t, step, loss_fn = beam_problem()
    assert np.array_equal(fx["mu_scale"], sc.extra["mu_scale"].astype(np.float32))
    q0 = model.particle_q.clone()
    v0 = torch.zeros_like(q0)
    steps = sc.frames * sc.substeps
    every = sc.extra["checkpoint_every"] * sc.substeps
    loss, _, dv0, (gs,) = checkpointed_gradient(step, q0, v0, steps, every, loss_fn, params=(s_t,))
    gs, dv0 = to_np(gs), to_np(dv0)
    got = np.array([gs[i] if k == 0 else dv0[i, a] for k, i, a in zip(fx["kind"], fx["index"], fx["axis"])])
    fd = fx["fd"]
    np.testing.assert_allclose(float(loss), float(fx["loss"]), rtol=1e-3)
    assert np.linalg.norm(got - fd) <= 1e-3 * np.linalg.norm(fd), (got, fd)
    np.testing.assert_allclose(got, fd, rtol=1e-3, atol=1e-3 * np.abs(fd).max())


def test_beam_backward_costs_at_most_three_forwards():
    """The adjoint pass (segment recomputation excluded) against one recorded forward rollout."""
    sc, model, s_t, step, loss_fn = beam_problem()
    q0 = model.particle_q.clone()
    steps = sc.frames * sc.substeps

    def forward():
        q, v = q0, torch.zeros_like(q0).requires_grad_(True)
        for k in range(steps):
            q, v = step(q, v, k)
        return loss_fn(q, v)

    forward().backward()  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = forward()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    loss.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    assert (t2 - t1) <= 3.0 * (t1 - t0), (t1 - t0, t2 - t1)


def test_backward_after_a_matrix_refresh_raises():
    """A tape recorded before refresh_tangent cannot be differentiated (differentiation.py:375-376)."""
    x, tets, mats, mass, scale, fixed = small_beam()
    model, solver, _ = make_pair(x, mass, tets=tets, tet_materials=mats, fixed=fixed, dt=1.0 / 240.0,
                                 with_oracle=False)
    diff = DifferentiableSolver(solver)
    v = torch.zeros_like(model.particle_q).requires_grad_(True)
    q1, v1 = diff.step(model.particle_q.clone(), v, solver.dt)
    solver.refresh_tangent(q1.detach().contiguous())
    with pytest.raises(RuntimeError, match="changed after recording"):
        q1.sum().backward()


def test_per_segment_refresh_matches_frozen_matrix_segments():
    """Checkpointed gradient with a tangent refresh at every segment start equals the product of the
    per-segment frozen-matrix gradients computed one segment at a time."""
    x, tets, mats, mass, scale, fixed = small_beam()
    dt = 1.0 / 240.0
    model, solver, _ = make_pair(x, mass, tets=tets, tet_materials=mats, fixed=fixed, dt=dt,
                                 linear_solver_maxiter=200, with_oracle=False)
    diff = DifferentiableSolver(solver, tolerance=1e-7, maxiter=200)
    q0 = model.particle_q.clone()
    v0 = torch.zeros_like(q0)

    def step(q, v, k):
        if k % 3 == 0:
            solver.refresh_tangent(q.detach().contiguous())
        return diff.step(q, v, dt)

    def loss_fn(q, v):
        return (q[:, 2] ** 2).sum() + 0.1 * (v ** 2).sum()

    _, dq_c, dv_c, _ = checkpointed_gradient(step, q0, v0, 9, 3, loss_fn)
    # the same chain by hand: forward to each segment start, then segment-wise VJPs from the end
    with torch.no_grad():
        starts, q, v = [], q0.clone(), v0.clone()
        for k in range(9):
            if k % 3 == 0:
                starts.append((q.clone(), v.clone()))
            q, v = step(q, v, k)
    qf, vf = q.clone().requires_grad_(True), v.clone().requires_grad_(True)
    qb, vb = torch.autograd.grad(loss_fn(qf, vf), (qf, vf))
    for seg in reversed(range(3)):
        qs = starts[seg][0].clone().requires_grad_(True)
        vs = starts[seg][1].clone().requires_grad_(True)
        q, v = qs, vs
        for k in range(3 * seg, 3 * seg + 3):
            q, v = step(q, v, k)
        qb, vb = torch.autograd.grad((q, v), (qs, vs), grad_outputs=(qb, vb))
    np.testing.assert_allclose(to_np(dq_c), to_np(qb), rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(to_np(dv_c), to_np(vb), rtol=1e-6, atol=1e-9)


def test_load_optimization_recovers_the_tip_load():
    """Fit a tip load from a cantilever's final shape by gradient descent through the
    differentiable step (tests/test_solver.py:424-429, tests/diffsim_optimize.py): the bundled
    12-node Tet4 cantilever, x = 0 nodes massless and restored after every substep, 12 substeps
    of 0.01 s, loss 1e4 * mean |q - target|^2; secant step sizes with a backtracking check."""
    from fixtures import mesh

    points, tets = mesh("tet_cantilever")
    b = FEMBuilder(gravity=(0.0, 0.0, 0.0))
    b.add_soft_mesh(pos=(0.0, 0.0, 0.0), rot=(0.0, 0.0, 0.0, 1.0), scale=1.0, vel=(0.0, 0.0, 0.0),
                    vertices=points, indices=tets.reshape(-1), density=100.0, k_mu=500.0, k_lambda=1000.0,
                    k_damp=0.1)
    for i, p in enumerate(b.particle_q):
        if abs(p[0]) < 1.0e-8:
            b.particle_mass[i] = 0.0
    model = b.finalize(DEVICE)
    dt = 0.01
    solver = SolverFEM(model, dt=dt, linear_solver_maxiter=64, solver_type="cg", preconditioner_type="block_diag",
                       min_stretch=-1.0, self_contact_ke=0.0)
    diff = DifferentiableSolver(solver)
    rest = model.particle_q.clone()
    support = (model.particle_inv_mass == 0.0)[:, None]
    x0 = rest[:, 0].cpu().numpy()
    weights = torch.as_tensor((x0 > 0.199) / (x0 > 0.199).sum(), dtype=torch.float32, device=DEVICE)

    def final_q(amplitude):
        q, v = rest.clone(), torch.zeros_like(rest)
        for _ in range(12):
            force = torch.stack([torch.zeros_like(weights), torch.zeros_like(weights), amplitude * weights], 1)
            raw_q, raw_v = diff.step(q, v, dt, external_forces=force)
            q = torch.where(support, rest, raw_q)
            v = torch.where(support, torch.zeros_like(raw_v), raw_v)
        return q

    def loss_of(q):
        return 1.0e4 * ((q - target) ** 2).sum() / q.shape[0]

    with torch.no_grad():
        target = final_q(torch.tensor(-0.2, device=DEVICE))
    amplitude = torch.tensor(-0.06, device=DEVICE, requires_grad=True)
    history, previous, accepted_updates = [], None, 0
    for iteration in range(16):
        loss = loss_of(final_q(amplitude))
        value = float(loss.detach())
        history.append(value)
        if iteration == 15 or value < 1.0e-11:
            break
        (gradient,) = torch.autograd.grad(loss, amplitude)
        gradient, current = float(gradient), float(amplitude.detach())
        assert np.isfinite(gradient)
        rate = 0.08 / max(abs(gradient), 1.0e-12)
        if previous is not None:
            change = current - previous[0]
            curvature = (gradient - previous[1]) / change if abs(change) > 1.0e-10 else 0.0
            if curvature > 0.0:
                rate = 1.0 / curvature
        accepted = False
        for _ in range(12):
            candidate = current - rate * gradient
            with torch.no_grad():
                trial = float(loss_of(final_q(torch.tensor(candidate, device=DEVICE))))
            if trial < value:
                previous = current, gradient
                with torch.no_grad():
                    amplitude.fill_(candidate)
                accepted_updates += 1
                accepted = True
                break
            rate *= 0.5
        if not accepted:
            break
    assert accepted_updates > 0
    assert history[-1] < 0.01 * history[0]
    assert abs(float(amplitude.detach()) - (-0.2)) < 0.01
    tip = torch.as_tensor(x0 > 0.199, device=DEVICE)
    assert abs(float((target - rest)[tip, 2].mean())) > 1.0e-5
