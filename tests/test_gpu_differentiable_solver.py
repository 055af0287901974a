"""``SolverFEM(model, differentiable=True)``: the reference's taped step, recorded by torch autograd
(``-m gpu``).

Restates the reference's differentiable-mode tests (``tests/test_solver.py``): multistep state and
force derivatives against central differences of the same solver (``:262-309``, tolerance rtol 0.015
/ atol 1e-4 as there), reuse of the solver for a second identical rollout, the h/2 force derivative of a
zero right-hand side (``:322-331``), the dense-solve step (``:240-260``) and the argument rejections
(``solver.py:250-251``; ``differentiation.py:236-296``).
"""

import numpy as np
import pytest
import torch
from fixtures import DT, cube_arrays
from gpu_helpers import DEVICE, make_pair, rounded, tensor, to_np

from newton_solver_fem_gb300 import FEMBuilder, SolverFEM, model_from_arrays

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _cuda(cuda_device):
    yield


def cube_model(kind="tet", gravity=(0.0, 0.0, 0.0)):
    x, el, mass, mats = cube_arrays(kind)
    if kind == "tet":
        return model_from_arrays(rounded(x), rounded(mass), tets=el, tet_materials=mats, radius=0.004,
                                 gravity=gravity, device=DEVICE)
    return model_from_arrays(rounded(x), rounded(mass), hexes=el, hex_materials=mats, radius=0.004, gravity=gravity,
                             device=DEVICE)


def make_solver(model, **options):
    """tests/test_solver.py:53-64."""
    args = dict(dt=DT, differentiable=True, linear_solver_maxiter=128, solver_type="cg",
                preconditioner_type="block_diag", self_contact_ke=0.0, min_stretch=-1.0)
    args.update(options)
    return SolverFEM(model, **args)


def objective(q, v):
    """tests/test_solver.py:19-24: sum_i q_i . ((i+1)/N, 0.13, -0.41) + 0.03 |v_i|^2, in float64."""
    n = q.shape[0]
    w = torch.stack([torch.arange(1, n + 1, device=q.device, dtype=torch.float64) / n,
                     torch.full((n,), 0.13, device=q.device, dtype=torch.float64),
                     torch.full((n,), -0.41, device=q.device, dtype=torch.float64)], dim=1)
    return (q.double() * w).sum() + 0.03 * (v.double() ** 2).sum()


def evaluate(model, solver, q, v, forces, record=True):
    """tests/test_solver.py:98-133: a rollout of len(forces) steps, optionally recorded, and its loss."""
    steps = len(forces)
    states = [model.state() for _ in range(steps + 1)]
    states[0].particle_q = tensor(q).requires_grad_(record)
    states[0].particle_qd = tensor(v).requires_grad_(record)
    inputs = [tensor(f).requires_grad_(record) for f in forces]
    with torch.set_grad_enabled(record):
        for i in range(steps):
            solver.step(states[i], states[i + 1], None, None, solver.dt, external_forces=inputs[i])
        loss = objective(states[-1].particle_q, states[-1].particle_qd)
    if record:
        loss.backward()
    return float(loss), states, inputs


@pytest.mark.parametrize("kind", ["tet", "hex"])
def test_multistep_state_force_gradients_and_reuse(kind):
    model = cube_model(kind)
    solver = make_solver(model)
    q = to_np(model.particle_q)
    q[:, 0] *= 1.03
    velocity = np.tile((0.02, -0.01, 0.03), (len(q), 1)).astype(np.float32)
    forces = np.zeros((3, *q.shape), dtype=np.float32)
    forces[:, -1, 2] = -0.02
    direction = np.random.default_rng(1).normal(size=q.shape).astype(np.float32)
    direction /= np.linalg.norm(direction)
    base, states, force_arrays = evaluate(model, solver, q, velocity, forces)
    exact = [float(np.sum(to_np(states[0].particle_q.grad) * direction)),
             float(np.sum(to_np(states[0].particle_qd.grad) * direction)),
             float(sum(np.sum(to_np(f.grad) * direction) for f in force_arrays))]
    for index, epsilons in enumerate(((2e-4, 1e-4), (2e-3, 1e-3), (2e-3, 1e-3))):
        for epsilon in epsilons:
            plus = [q.copy(), velocity.copy(), forces.copy()]
            minus = [q.copy(), velocity.copy(), forces.copy()]
            plus[index] += epsilon * direction
            minus[index] -= epsilon * direction
            numeric = (evaluate(model, solver, *plus, record=False)[0]
                       - evaluate(model, solver, *minus, record=False)[0]) / (2 * epsilon)
            np.testing.assert_allclose(exact[index], numeric, rtol=0.015, atol=1e-4,
                                       err_msg=f"{kind} input={index} epsilon={epsilon}")
    repeated, second, _ = evaluate(model, solver, q, velocity, forces)
    assert abs(base - repeated) < 1e-6
    np.testing.assert_allclose(to_np(second[0].particle_q.grad), to_np(states[0].particle_q.grad), rtol=2e-6,
                               atol=1e-6)
    residuals = solver.check()
    assert residuals["forward_relative_residual"] <= 2e-5 and residuals["backward_relative_residual"] <= 2e-5


def test_zero_rhs_has_nonzero_force_derivative():
    """A free 2 kg particle at rest: d v_x / d f_ext = h / 2 through the taped step."""
    b = FEMBuilder(gravity=(0.0, 0.0, 0.0))
    b.add_particle((0, 0, 1), (0, 0, 0), mass=2.0)
    model = b.finalize(DEVICE)
    solver = make_solver(model)
    initial, output = model.state(), model.state()
    external = torch.zeros((1, 3), device=DEVICE, requires_grad=True)
    solver.step(initial, output, None, None, DT, external_forces=external)
    output.particle_qd[:, 0].double().sum().backward()
    np.testing.assert_allclose(to_np(external.grad), [[DT / 2, 0, 0]], atol=1e-8)


def test_differentiable_step_matches_dense_solve_and_preserves_inputs():
    """tests/test_solver.py:240-260 with the default differentiable solver: every solve is a checked
    solve from zero, equal to the dense solution."""
    model = cube_model()
    solver = make_solver(model)
    initial, output = model.state(), model.state()
    q = to_np(model.particle_q).astype(np.float32)
    q[-1, 2] -= 0.001
    initial.particle_q.copy_(tensor(q))
    velocity = np.random.default_rng(2).normal(0, 0.03, q.shape).astype(np.float32)
    initial.particle_qd.copy_(tensor(velocity))
    force = np.zeros_like(q)
    force[-1] = (0.1, 0.05, -0.2)
    external = tensor(force)
    mass = np.repeat(to_np(model.particle_mass), 3)
    matrix = solver.A_bsr.dense()
    st = model.state()
    st.particle_q, st.particle_qd = initial.particle_q, initial.particle_qd
    elastic = to_np(solver.eval_tetrahedral_forces(model, None, st))
    rhs = DT * (force + elastic).flatten() - matrix @ velocity.flatten() + mass * velocity.flatten()
    increment = np.linalg.solve(matrix, rhs).reshape(q.shape)
    solver.step(initial, output, None, None, DT, external_forces=external)
    np.testing.assert_allclose(to_np(output.particle_qd), velocity + increment, rtol=3e-4, atol=3e-6)
    np.testing.assert_allclose(to_np(output.particle_q), q + DT * (velocity + increment), rtol=1e-6, atol=1e-7)
    np.testing.assert_array_equal(to_np(initial.particle_q), q)
    np.testing.assert_array_equal(to_np(initial.particle_qd), velocity)
    np.testing.assert_array_equal(to_np(external), force)


def test_differentiable_mode_rejections():
    model = cube_model()
    with pytest.raises(ValueError, match="fixed_particle_indices"):
        make_solver(model, fixed_particle_indices=[0])
    solver = make_solver(model)
    s0, s1 = model.state(), model.state()
    with pytest.raises(ValueError, match="timestep"):
        solver.step(s0, s1, None, None, 2 * DT)
    with pytest.raises(NotImplementedError, match="analytic ground"):
        solver.step(s0, s1, None, object(), DT)
    with pytest.raises(ValueError, match="unique input/output"):
        solver.step(s0, s0, None, None, DT)
    contact = make_solver(cube_model(), self_contact_ke=1.0e3)  # the reference's default self contact
    with pytest.raises(NotImplementedError, match="particle/surface"):
        contact.step(model.state(), model.state(), None, None, DT)


def test_unconverged_differentiable_solve_raises_unless_deferred():
    """A checked solve that cannot meet the residual budget raises (differentiation.py:263-272); with
    deferred checks the step returns and check() raises later."""
    model = cube_model()
    solver = make_solver(model, linear_solver_maxiter=1)
    s0, s1 = model.state(), model.state()
    s0.particle_qd.copy_(torch.randn_like(s0.particle_qd) * 0.05)
    with pytest.raises(RuntimeError, match="did not converge"):
        solver.step(s0, s1, None, None, DT)
    deferred = make_solver(model, linear_solver_maxiter=1, defer_differentiation_checks=True)
    deferred.step(s0, s1, None, None, DT)
    with pytest.raises(RuntimeError, match="did not converge"):
        deferred.check()
