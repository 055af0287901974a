"""Device-side differentiable rollouts and per-element material VJPs (``-m gpu``).

``fem_rollout_segment`` / ``fem_adjoint_segment`` run whole checkpoint segments on
the device; they must give the gradients of the per-substep autograd path
(``_Substep``), whose float64-difference checks live in ``test_gpu_adjoint.py``,
and meet the differentiable beam's bar on their own: float64 central differences
within 1e-3 relative, at no more than 3x the plain ``SolverFEM.step`` rollout.
``fem_force_vjp_materials`` gives dL/d(mu, lambda, k_d) per element, checked
against float64 central differences of the oracle's forces.
"""

import time
from pathlib import Path

import numpy as np
import pytest
import torch
from gpu_helpers import DEVICE, make_pair, rounded, scene_pair, tensor, to_np

from newton_solver_fem_gb300 import _lib, scenes
from newton_solver_fem_gb300.adjoint import (DeviceRollout, DifferentiableSolver, checkpointed_gradient,
                                             device_checkpointed_gradient)
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).with_name("golden")


@pytest.fixture(autouse=True)
def _cuda(cuda_device):
    yield


def small_beam(nx=4, seed=0, k_damp=0.0):
    x, tets, mats, mass = scenes.tet_block(nx, 1, 1, 0.05, (0, 0, 0), 1.0e5, 0.45, 1000.0, k_damp=k_damp)
    rng = np.random.default_rng(seed)
    scale = rng.uniform(0.8, 1.2, size=len(tets)).astype(np.float32)
    fixed = np.nonzero(np.isclose(x[:, 0], 0.0))[0].astype(np.int32)
    return x, tets, mats, mass, scale, fixed


def _beam_setup(tol=1e-7, maxiter=200, **kw):
    x, tets, mats, mass, scale, fixed = small_beam(**kw)
    dt = 1.0 / 240.0
    model, solver, _ = make_pair(x, mass, tets=tets, tet_materials=mats, gravity=(0, 0, -9.81), fixed=fixed, dt=dt,
                                 linear_solver_maxiter=maxiter, with_oracle=False)
    diff = DifferentiableSolver(solver, tolerance=tol, maxiter=maxiter)
    s_t = tensor(scale).requires_grad_(True)
    diff.set_mu_scale(s_t)
    solver.refresh_tangent(model.particle_q.clone())  # A at the nominal scales, frozen from here on
    return model, solver, diff, s_t, dt


def test_device_gradient_equals_the_autograd_tape():
    """12 substeps, checkpoints every 4: gradients wrt q0, v0, a held load and the shear scales from the
    device segments equal the per-substep autograd path (same kernels, same order)."""
    model, solver, diff, s_t, dt = _beam_setup()
    rng = np.random.default_rng(5)
    P = model.particle_count
    q0 = model.particle_q.clone()
    v0 = tensor(rng.normal(0, 0.02, (P, 3)))
    ext = tensor(rng.normal(0, 0.01, (P, 3))).requires_grad_(True)
    target = q0.mean(0) - torch.tensor([0.0, 0.0, 0.01], device=DEVICE)

    def loss_fn(q, v):
        return ((q.mean(0) - target) ** 2).sum() + 0.1 * (v ** 2).sum()

    def step(q, v, k):
        return diff.step(q, v, dt, external_forces=ext, mu_scale=s_t)

    loss_h, dq_h, dv_h, (gs_h, ge_h) = checkpointed_gradient(step, q0, v0, 12, 4, loss_fn, params=(s_t, ext))
    for graphs in (False, True):
        loss_d, g = device_checkpointed_gradient(diff, q0, v0, 12, 4, loss_fn, external_forces=ext, mu_scale=s_t,
                                                 graphs=graphs)
        np.testing.assert_allclose(loss_d.item(), loss_h.item(), rtol=1e-6)
        for got, want in ((g["q0"], dq_h), (g["v0"], dv_h), (g["mu_scale"], gs_h), (g["external_forces"], ge_h)):
            got, want = to_np(got), to_np(want)
            np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-5 * np.abs(want).max())


def test_store_all_equals_checkpoint_recomputation():
    """Keeping every substep state (no recomputation) gives the recomputation's gradients bit for bit."""
    model, solver, diff, s_t, dt = _beam_setup()
    q0 = model.particle_q.clone()
    v0 = torch.zeros_like(q0)

    def loss_fn(q, v):
        return (q[:, 2] ** 2).sum() + 0.1 * (v ** 2).sum()

    _, g_re = device_checkpointed_gradient(diff, q0, v0, 10, 4, loss_fn, mu_scale=s_t)
    _, g_all = device_checkpointed_gradient(diff, q0, v0, 10, 4, loss_fn, mu_scale=s_t, store_all=True)
    for k in ("q0", "v0", "mu_scale"):
        np.testing.assert_array_equal(to_np(g_re[k]), to_np(g_all[k]))


def test_per_segment_refresh_matches_the_host_schedule():
    """A tangent refresh at every segment start (a segment is one frame) gives the host path's gradients,
    with recomputation and with every state kept."""
    model, solver, diff, s_t, dt = _beam_setup()
    q0 = model.particle_q.clone()
    v0 = torch.zeros_like(q0)

    def loss_fn(q, v):
        return (q[:, 2] ** 2).sum() + 0.1 * (v ** 2).sum()

    def step(q, v, k):
        if k % 3 == 0:
            solver.refresh_tangent(q.detach().contiguous())
        return diff.step(q, v, dt, mu_scale=s_t)

    _, dq_h, dv_h, (gs_h,) = checkpointed_gradient(step, q0, v0, 9, 3, loss_fn, params=(s_t,))
    for store_all in (False, True):
        _, g = device_checkpointed_gradient(diff, q0, v0, 9, 3, loss_fn, mu_scale=s_t, refresh=True,
                                            store_all=store_all)
        for got, want in ((g["q0"], dq_h), (g["v0"], dv_h), (g["mu_scale"], gs_h)):
            got, want = to_np(got), to_np(want)
            np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-5 * np.abs(want).max())


def _beam():
    sc = scenes.tet_beam()
    model, solver, _ = make_pair(sc.x, sc.mass, tets=sc.tets, tet_materials=sc.tet_materials, fixed=sc.fixed,
                                 dt=sc.dt, linear_solver_maxiter=sc.maxiter, linear_solver_tolerance=1.0e-8,
                                 with_oracle=False)
    diff = DifferentiableSolver(solver, tolerance=1.0e-8, maxiter=sc.maxiter)
    s_t = tensor(sc.extra["mu_scale"])
    diff.set_mu_scale(s_t)
    solver.refresh_tangent(model.particle_q.clone())
    tip = torch.as_tensor(sc.extra["tip_nodes"], device=DEVICE, dtype=torch.long)
    target = tensor(sc.extra["target"])

    def loss_fn(q, v):
        return ((q[tip].mean(0) - target) ** 2).sum()

    return sc, model, solver, diff, s_t, loss_fn


def test_device_beam_gradient_matches_fp64_differences():
    """The differentiable beam: 120 frames x 4 substeps, checkpoints every 10 frames, device segments
    replayed from a captured graph, against float64 central differences (eps 1e-3) at 1e-3."""
    fx = np.load(GOLDEN / "beam_fd.npz")
    sc, model, solver, diff, s_t, loss_fn = _beam()
    q0 = model.particle_q.clone()
    v0 = torch.zeros_like(q0)
    steps = sc.frames * sc.substeps
    every = sc.extra["checkpoint_every"] * sc.substeps
    loss, g = device_checkpointed_gradient(diff, q0, v0, steps, every, loss_fn, mu_scale=s_t)
    gs, dv0 = to_np(g["mu_scale"]), to_np(g["v0"])
    got = np.array([gs[i] if k == 0 else dv0[i, a] for k, i, a in zip(fx["kind"], fx["index"], fx["axis"])])
    fd = fx["fd"]
    np.testing.assert_allclose(float(loss), float(fx["loss"]), rtol=1e-3)
    assert np.linalg.norm(got - fd) <= 1e-3 * np.linalg.norm(fd), (got, fd)
    np.testing.assert_allclose(got, fd, rtol=1e-3, atol=1e-3 * np.abs(fd).max())


def test_device_beam_gradient_costs_at_most_three_plain_rollouts():
    """The checkpointed gradient (forward with checkpoints + per-segment recomputation + reverse pass)
    against the same 480 substeps through SolverFEM.step replayed from a captured frame graph."""
    sc, model, solver, diff, s_t, loss_fn = _beam()
    q0 = model.particle_q.clone()
    v0 = torch.zeros_like(q0)
    steps = sc.frames * sc.substeps
    every = sc.extra["checkpoint_every"] * sc.substeps
    a, b = model.state(), model.state()
    stream = torch.cuda.Stream()

    def plain_frame():
        x, y = a, b
        for _ in range(sc.substeps):
            solver.step(x, y, None, None, sc.dt)
            x, y = y, x

    with torch.cuda.stream(stream):
        plain_frame()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            plain_frame()
    # a second handle over the same beam recomputes segments concurrently with the reverse pass
    _, _, _, diff2, _, _ = _beam()
    diff2.set_mu_scale(s_t)
    ro = DeviceRollout(diff, steps, every, overlap=diff2)
    assert ro.overlap is not None

    def plain():
        with torch.cuda.stream(stream):
            for _ in range(sc.frames):
                graph.replay()

    def gradient():
        device_checkpointed_gradient(diff, q0, v0, steps, every, loss_fn, mu_scale=s_t, rollout=ro)

    def best(fn, n=3):
        out = []
        for _ in range(n):
            torch.cuda.synchronize()
            t = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            out.append(time.perf_counter() - t)
        return min(out)

    plain(), gradient()  # warm-up (graph capture of the segment)
    t_plain, t_grad = best(plain), best(gradient)
    assert t_grad <= 3.0 * t_plain, (t_plain, t_grad)


def test_overlapped_recomputation_gives_the_in_line_gradients():
    """Recomputing segments on a second handle and stream gives bit-identical gradients."""
    sc, model, solver, diff, s_t, loss_fn = _beam()
    _, _, _, diff2, _, _ = _beam()
    diff2.set_mu_scale(s_t)
    q0 = model.particle_q.clone()
    v0 = torch.zeros_like(q0)
    steps, every = 10 * sc.substeps, 2 * sc.substeps
    _, g_line = device_checkpointed_gradient(diff, q0, v0, steps, every, loss_fn, mu_scale=s_t)
    ro = DeviceRollout(diff, steps, every, overlap=diff2)
    assert ro.overlap is not None
    for _ in range(2):  # the second call replays the graphs captured by the first
        _, g_over = device_checkpointed_gradient(diff, q0, v0, steps, every, loss_fn, mu_scale=s_t, rollout=ro)
        for k in ("q0", "v0", "mu_scale"):
            np.testing.assert_array_equal(to_np(g_over[k]), to_np(g_line[k]))


def _material_vjp(solver, q, v, g):
    lib = _lib.load()
    z = torch.zeros_like(q)
    T, H = solver.model.tet_count, solver.hex_count
    tb = torch.zeros((T, 3), device=DEVICE) if T else None
    hb = torch.zeros((H, 3), device=DEVICE) if H else None
    _lib.check(lib.fem_force_vjp_materials(solver._handle, q.data_ptr(), v.data_ptr(), None,
                                           solver.model.gravity.data_ptr(), g.data_ptr(), z.data_ptr(),
                                           torch.zeros_like(q).data_ptr(), None, None,
                                           None if tb is None else tb.data_ptr(), None if hb is None else hb.data_ptr(),
                                           torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return None if tb is None else to_np(tb), None if hb is None else to_np(hb)


@pytest.mark.parametrize("kind", ["tet", "hex"])
def test_material_vjp_matches_differences(kind):
    """dL/d(mu, lambda, k_d) per element of L = g . f(q, v; materials), against float64 central
    differences of the oracle's element forces (Rayleigh damping on, deformed and moving state)."""
    rng = np.random.default_rng(17)
    if kind == "tet":
        x, el, mats, mass = scenes.tet_block(3, 2, 2, 0.05, (0, 0, 0), 1.0e5, 0.45, 1000.0, k_damp=3.0)
        cell = 0.05
    else:
        x, el, mats, mass = scenes.hex_block(3, 2, 2, 0.01, (0, 0, 0), 5.0e5, 0.4, 1100.0, k_damp=2.0)
        cell = 0.01
    # per-element materials vary so that every element's gradient is distinct
    mats = (mats * rng.uniform(0.7, 1.3, size=mats.shape)).astype(np.float32)
    if kind == "tet":
        model, solver, oracle = make_pair(x, mass, tets=el, tet_materials=mats, gravity=(0, 0, 0))
    else:
        model, solver, oracle = make_pair(x, mass, hexes=el, hex_materials=mats, gravity=(0, 0, 0))
    q = rounded(oracle.rest + rng.normal(0, 0.03 * cell, x.shape))
    v = rounded(rng.normal(0, 0.05, x.shape))
    g = rounded(rng.normal(0, 1.0, x.shape))
    tb, hb = _material_vjp(solver, tensor(q), tensor(v), tensor(g))
    got = tb if kind == "tet" else hb
    base = (oracle.tet_materials if kind == "tet" else oracle.hex_materials).astype(np.float64).copy()
    term = (kind,)
    for col in range(3):
        d = np.zeros_like(base)
        d[:, col] = rng.normal(size=len(base)) * np.abs(base[:, col]).mean()
        eps = 1e-6
        vals = []
        for sgn in (1.0, -1.0):
            m = base + sgn * eps * d
            if kind == "tet":
                oracle.tet_materials = m
            else:
                oracle.hex_materials = m
            vals.append(float(np.sum(g * oracle.forces(q, v, terms=term)[kind])))
        if kind == "tet":
            oracle.tet_materials = base
        else:
            oracle.hex_materials = base
        fd = (vals[0] - vals[1]) / (2 * eps)
        exact = float(np.sum(got * d))
        assert abs(exact - fd) <= 1e-3 * abs(fd) + 1e-9, (kind, col, exact, fd)


def test_material_gradient_through_a_rollout_matches_differences():
    """Accumulated dL/d(mu, lambda, k_d) of the device reverse pass over 4 substeps (matrix frozen at the
    nominal materials, forces at the perturbed ones) against float64 central differences."""
    x, tets, mats, mass, scale, fixed = small_beam(k_damp=2.0)
    dt = 1.0 / 240.0
    model, solver, oracle = make_pair(x, mass, tets=tets, tet_materials=mats, gravity=(0, 0, -9.81), fixed=fixed,
                                      dt=dt, linear_solver_maxiter=200)
    oracle = O.OracleFEM(oracle.rest, oracle.mass, tets=tets, tet_poses=oracle.tet_poses, tet_materials=mats,
                         gravity=(0, 0, -9.81), fixed=fixed, dt=dt, maxiter=400, tolerance=1e-13)
    diff = DifferentiableSolver(solver, tolerance=1e-7, maxiter=200)
    solver.refresh_tangent(model.particle_q.clone())
    rng = np.random.default_rng(9)
    q0 = rounded(oracle.rest + rng.normal(0, 1e-3, x.shape))
    q0[fixed] = oracle.rest[fixed]
    v0 = rounded(rng.normal(0, 0.02, x.shape))
    v0[fixed] = 0.0
    w = rng.normal(size=x.shape)
    wt = torch.tensor(w, device=DEVICE, dtype=torch.float32)
    _, g = device_checkpointed_gradient(diff, tensor(q0), tensor(v0), 4, 2, lambda q, v: (wt * q).sum(),
                                        materials=True)
    got = to_np(g["tet_materials"])
    base = mats.astype(np.float64)
    for col in range(3):
        d = np.zeros_like(base)
        d[:, col] = rng.normal(size=len(base)) * np.abs(base[:, col]).mean()
        eps = 1e-5
        vals = []
        for sgn in (1.0, -1.0):
            oracle.tet_materials = base + sgn * eps * d
            q, v = q0.copy(), v0.copy()
            oracle.dv[:] = 0.0
            for _ in range(4):
                oracle.dv[:] = 0.0
                q, v, _ = oracle.step(q, v, dt)
            vals.append(float(np.sum(w * q)))
        oracle.tet_materials = base
        fd = (vals[0] - vals[1]) / (2 * eps)
        exact = float(np.sum(got * d))
        assert abs(exact - fd) <= 1e-3 * abs(fd) + 1e-9, (col, exact, fd)


def test_rollout_rejects_a_timestep_other_than_the_assembled_one():
    model, solver, diff, s_t, dt = _beam_setup()
    q = model.particle_q.clone()
    states = torch.zeros((3, model.particle_count, 3), device=DEVICE)
    code = _lib.load().fem_rollout_segment(solver._handle, q.data_ptr(), q.data_ptr(), None, 2, None, None, None,
                                           dt * 2, 1e-7, 10, 0, 0, states.data_ptr(), states.data_ptr(), None,
                                           torch.cuda.current_stream().cuda_stream)
    assert code == _lib.FEM_ERR_BAD_ARG
