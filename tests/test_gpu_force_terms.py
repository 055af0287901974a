"""Triangle membranes, spring bend torque, particle-particle contact and soft-rigid contacts on
the GPU (``-m gpu``) against the CPU oracle.

Reference kernels (``src/newton_solver_fem/_src/solvers/fem/``): ``eval_triangles`` and
``build_system_matrix_tri_kernel`` (kernels.py:876-1012), ``eval_springs_linear_and_torque``
(kernels.py:221-291), ``eval_particle_forces`` (kernels.py:1036-1114) and ``eval_soft_contacts``
(kernels.py:1198-1261), accumulated in solver.py:571-589 order.  Tolerances: forces 2e-5 of the
largest entry (float32 kernels vs the float64 oracle); one substep with a fixed CG iteration count
1e-4 relative L2; adjoint directional derivatives 1e-3 relative (central differences of the
oracle).  Contact sums run in a fixed order, so repeated evaluations are bit-identical.
"""

import numpy as np
import pytest
import torch
from gpu_helpers import DEVICE, face_triangles, make_pair, rel_l2, rounded, tensor, to_np

from newton_solver_fem_gb300 import Contacts, _lib, scenes
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu

DT = 1.0 / 600.0


@pytest.fixture(autouse=True)
def _cuda(cuda_device):
    yield


def plate(nx=12, ny=9, h=0.02, z=0.3, seed=0):
    """A flat membrane of (nx x ny) cells, two triangles each, with random materials."""
    g = np.stack(np.meshgrid(np.arange(nx + 1) * h, np.arange(ny + 1) * h, indexing="ij"), -1).reshape(-1, 2)
    x = np.column_stack([g, np.full(len(g), z)])
    tris = face_triangles(x, 2, z)
    rng = np.random.default_rng(seed)
    mats = np.column_stack([rng.uniform(10, 50, len(tris)), rng.uniform(20, 80, len(tris)),
                            rng.uniform(0, 0.05, len(tris)), rng.uniform(0, 0.5, len(tris)),
                            rng.uniform(0, 0.5, len(tris))]).astype(np.float32)
    return x, tris, mats


def set_state(model, q, v):
    s = model.state()
    s.particle_q.copy_(tensor(q))
    s.particle_qd.copy_(tensor(v))
    return s


def close(got, want, rel=2e-5):
    np.testing.assert_allclose(got, want, rtol=0, atol=rel * max(np.abs(want).max(), 1e-30))


# ---------------------------------------------------------------- triangles


def test_triangle_forces_match_oracle_with_drag_and_lift():
    x, tris, mats = plate()
    model, solver, oracle = make_pair(x, np.full(len(x), 1e-3), tris=tris, tri_materials=mats)
    rng = np.random.default_rng(1)
    q = rounded(x + rng.normal(0, 2e-3, x.shape))
    v = rounded(rng.normal(0, 0.3, x.shape))
    f = to_np(solver.eval_triangle_forces(model, None, set_state(model, q, v)))
    close(f, oracle.forces(q, v, terms=("tri",))["tri"])


def test_triangle_rest_state_and_rigid_motion_give_no_membrane_force():
    x, tris, mats = plate(nx=4, ny=3)
    mats[:, 3:] = 0.0  # no drag / lift
    model, solver, oracle = make_pair(x, np.full(len(x), 1e-3), tris=tris, tri_materials=mats)
    c, s = np.cos(0.4), np.sin(0.4)
    R = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])
    q = rounded(x @ R.T + (0.1, -0.2, 0.05))
    f = to_np(solver.eval_triangle_forces(model, None, set_state(model, q, np.zeros_like(q))))
    scale = np.abs(oracle.forces(rounded(x * 1.05), np.zeros_like(x), terms=("tri",))["tri"]).max()
    assert np.abs(f).max() < 1e-4 * scale


def test_triangle_blocks_enter_the_matrix_in_the_reference_layout():
    """Lumped h^2 (mu + lambda) A_rest / 3 blocks sit between the springs and the tets: [P | 2S | 3Tri | 16T]."""
    xt, tets, mt, mass = scenes.tet_block(3, 2, 1, 0.05, (0.0, 0.0, 0.0), 1.0e5, 0.45, 1000.0)
    tris = face_triangles(xt, 2, 0.05)
    tm = np.tile(np.array([[30.0, 50.0, 0.03, 0.0, 0.0]], np.float32), (len(tris), 1))
    springs = np.array([[0, 5], [2, 7]], np.int32)
    model, solver, oracle = make_pair(xt, mass, tets=tets, tet_materials=mt, tris=tris, tri_materials=tm,
                                      springs=springs, spring_ke=np.float32([40, 50]), spring_kd=np.float32([0.2, 0.1]))
    rows, cols, vals = (to_np(t) for t in solver._triplets())
    orow, ocol, oval = oracle.triplets(oracle.rest, DT)
    P, S, Tri = len(xt), len(springs), len(tris)
    np.testing.assert_array_equal(rows, orow)
    np.testing.assert_array_equal(cols, ocol)
    region = slice(P + 2 * S, P + 2 * S + 3 * Tri)
    np.testing.assert_allclose(vals[region], oval[region], rtol=1e-6)
    np.testing.assert_allclose(solver.A_bsr.dense(), oracle.dense(), rtol=1e-5, atol=1e-6 * np.abs(oracle.dense()).max())


def test_triangle_substep_matches_oracle_fixed_iterations():
    x, tris, mats = plate(nx=10, ny=6)
    fixed = np.nonzero(np.isclose(x[:, 0], 0.0))[0].astype(np.int32)
    rng = np.random.default_rng(3)
    vel = rounded(rng.normal(0, 0.1, x.shape))
    vel[fixed] = 0.0
    model, solver, oracle = make_pair(x, np.full(len(x), 2e-3), tris=tris, tri_materials=mats, fixed=fixed,
                                      velocity=vel, linear_solver_maxiter=12, linear_solver_tolerance=1e-30)
    load = rounded(rng.normal(0, 0.01, x.shape))
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, DT, external_forces=tensor(load))
    _, v_ref, rhs = oracle.step(oracle.rest, vel, DT, external=load, fixed_iterations=12)
    assert rel_l2(to_np(s0.particle_f), rhs) < 1e-5
    assert rel_l2(to_np(solver.velocity_increment), oracle.dv) < 1e-4
    assert rel_l2(to_np(s1.particle_qd), v_ref) < 1e-4


# ---------------------------------------------------------------- bend torque


def spring_chain(n=24, seed=4):
    rng = np.random.default_rng(seed)
    x = np.cumsum(rng.normal(0, 0.02, (n, 3)) + (0.03, 0.0, 0.0), axis=0)
    springs = np.array([(i, i + 1) for i in range(n - 1)] + [(i, i + 2) for i in range(0, n - 2, 3)], np.int32)
    lo, hi = springs[:, 0], springs[:, 1]
    d = x[hi] - x[lo]
    rest_dir = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rest_dir[3] = 0.0  # a torque-free spring
    return x, springs, rest_dir


def test_spring_torque_forces_match_oracle():
    x, springs, rest_dir = spring_chain()
    S = len(springs)
    rng = np.random.default_rng(6)
    model, solver, oracle = make_pair(x, np.full(len(x), 0.01), springs=springs, spring_ke=np.full(S, 80.0, np.float32),
                                      spring_kd=np.full(S, 0.3, np.float32), spring_rest_direction=rest_dir,
                                      torque_stiffness=2.5, torque_damping=0.05)
    q = rounded(x + rng.normal(0, 4e-3, x.shape))
    q[5] = q[4] + rest_dir[4] * np.linalg.norm(x[5] - x[4])  # spring 4 (nodes 4, 5) at its rest direction: no torque
    q = rounded(q)
    v = rounded(rng.normal(0, 0.2, x.shape))
    f = to_np(solver.eval_spring_forces(model, set_state(model, q, v)))
    want = oracle.forces(q, v, terms=("spring",))["spring"]
    torque = O.spring_torque_forces(q, v, springs, rest_dir, 2.5, 0.05)
    assert np.abs(torque).max() > 0.05 * np.abs(want).max()  # the torque is a visible part of the term
    close(f, want)


# ---------------------------------------------------------------- particle-particle contact


def particle_cloud(P=3000, seed=7):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.0, 0.5, (P, 3))
    radius = rng.uniform(0.005, 0.01, P).astype(np.float32)
    flags = np.ones(P, np.int32)
    flags[rng.choice(P, P // 10, replace=False)] = 0
    v = rng.normal(0, 0.2, (P, 3))
    return x, radius, flags, v


def test_particle_contact_matches_all_pairs_and_is_deterministic():
    x, radius, flags, v = particle_cloud()
    coeffs = (1.0e3, 1.0e2, 1.0e2, 0.5, 0.002)
    model, solver, oracle = make_pair(x, np.full(len(x), 1e-3), radius=radius, flags=flags, particle_contact=coeffs,
                                      gravity=(0, 0, 0))
    q, vv = rounded(x), rounded(v)
    state = set_state(model, q, vv)
    f = solver.eval_particle_particle_forces(model, None, state)
    f2 = solver.eval_particle_particle_forces(model, None, state)
    torch.cuda.synchronize()
    assert torch.equal(f, f2)
    want = oracle.forces(q, vv, terms=("particle",))["particle"]
    assert (np.abs(want).sum(1) > 0).sum() > 100  # many particles in contact
    close(to_np(f), want)
    assert np.abs(to_np(f)[flags == 0]).max() == 0.0


def test_particle_contact_off_without_grid_radius_or_stiffness():
    x, radius, flags, v = particle_cloud(P=200)
    for kw in (dict(radius=0.0, particle_contact=(1e3, 1e2, 1e2, 0.5, 0.0)),
               dict(radius=radius, particle_contact=(0.0, 1e2, 1e2, 0.5, 0.0)),
               dict(radius=radius)):
        model, solver, _ = make_pair(x, np.full(len(x), 1e-3), gravity=(0, 0, 0), with_oracle=False, **kw)
        f = solver.eval_particle_particle_forces(model, None, set_state(model, rounded(x), rounded(v)))
        assert float(f.abs().max()) == 0.0


# ---------------------------------------------------------------- soft-rigid contacts


def contact_list(x, radius, capacity=64, count=50, seed=9):
    """Contacts against planes under random particles; some repeated particles, some invalid entries."""
    rng = np.random.default_rng(seed)
    c = Contacts(capacity, device=DEVICE)
    part = rng.integers(0, len(x), capacity).astype(np.int32)
    part[5:9] = part[4]  # several contacts on one particle
    part[10] = -1  # ignored entry
    normal = rng.normal(size=(capacity, 3))
    normal /= np.linalg.norm(normal, axis=1, keepdims=True)
    depth = rng.uniform(-0.5, 1.5, capacity) * np.asarray(radius)[part]  # about 3/4 penetrating
    body_pos = rounded(x[part] - normal * (np.asarray(radius)[part] - depth)[:, None])
    body_vel = rounded(rng.normal(0, 0.3, (capacity, 3)))
    c.soft_contact_count.fill_(count)
    c.soft_contact_particle.copy_(torch.tensor(part, device=DEVICE))
    c.soft_contact_body_pos.copy_(tensor(body_pos))
    c.soft_contact_body_vel.copy_(tensor(body_vel))
    c.soft_contact_normal.copy_(tensor(normal))
    host = (count, part, body_pos, body_vel, rounded(normal))
    return c, host


def test_soft_contacts_match_oracle_and_are_deterministic():
    x, radius, flags, v = particle_cloud(P=400, seed=2)
    model, solver, oracle = make_pair(x, np.full(len(x), 1e-3), radius=radius, gravity=(0, 0, 0),
                                      soft_contact=(2.0e3, 15.0, 8.0e2, 0.4))
    contacts, host = contact_list(rounded(x), radius)
    q, vv = rounded(x), rounded(v)
    state = set_state(model, q, vv)
    f = solver.eval_soft_contact_forces(model, state, contacts)
    f2 = solver.eval_soft_contact_forces(model, state, contacts)
    torch.cuda.synchronize()
    assert torch.equal(f, f2)
    want = oracle.forces(q, vv, terms=("soft_contact",), contacts=host)["soft_contact"]
    assert (np.abs(want).sum(1) > 0).sum() > 20
    close(to_np(f), want)
    contacts.soft_contact_count.fill_(0)  # entries past the device count are ignored
    assert float(solver.eval_soft_contact_forces(model, state, contacts).abs().max()) == 0.0


# ---------------------------------------------------------------- every term in one substep


def test_substep_with_every_force_term_matches_oracle():
    """Tets + membrane + torque springs + particle contact + soft contacts + ground + damping, fixed iterations."""
    xt, tets, mt, mass = scenes.tet_block(4, 3, 2, 0.05, (0.0, 0.0, 0.0245), 1.0e5, 0.45, 1000.0, k_damp=0.5)
    tris = face_triangles(xt, 2, xt[:, 2].max())
    tm = np.tile(np.array([[30.0, 50.0, 0.03, 0.3, 0.2]], np.float32), (len(tris), 1))
    top = np.nonzero(np.isclose(xt[:, 2], xt[:, 2].max()))[0]
    springs = np.stack([top[:-1], top[1:]], 1).astype(np.int32)
    S = len(springs)
    d = xt[springs[:, 1]] - xt[springs[:, 0]]
    rest_dir = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    radius = np.full(len(xt), 0.026, np.float32)  # axis neighbours (5 cm apart) overlap by 2 mm; bottom 1.5 mm in the ground
    rng = np.random.default_rng(12)
    vel = rounded(rng.normal(0, 0.1, xt.shape))
    model, solver, oracle = make_pair(
        xt, mass, tets=tets, tet_materials=mt, tris=tris, tri_materials=tm, springs=springs,
        spring_ke=np.full(S, 300.0, np.float32), spring_kd=np.full(S, 0.2, np.float32), spring_rest_direction=rest_dir,
        torque_stiffness=1.5, torque_damping=0.02, radius=radius, velocity=vel,
        particle_contact=(1.0e3, 1.0e2, 1.0e2, 0.5, 0.0), ground_plane=(0.0, 0.0, 1.0, 0.0), linear_damping=0.3,
        linear_solver_maxiter=10, linear_solver_tolerance=1e-30)
    q = rounded(xt + rng.normal(0, 4e-3, xt.shape))
    contacts, host = contact_list(q, radius, capacity=32, count=24, seed=13)
    s0, s1 = set_state(model, q, vel), model.state()
    solver.step(s0, s1, None, contacts, DT)
    terms = oracle.forces(q, vel, contacts=host)
    for key in ("tri", "particle", "soft_contact", "ground"):
        assert np.abs(terms[key]).max() > 0, key  # every term is active
    _, v_ref, rhs = oracle.step(q, vel, DT, fixed_iterations=10, contacts=host)
    assert rel_l2(to_np(s0.particle_f), rhs) < 1e-5
    assert rel_l2(to_np(solver.velocity_increment), oracle.dv) < 1e-4
    assert rel_l2(to_np(s1.particle_qd), v_ref) < 1e-4


# ---------------------------------------------------------------- adjoint of the new differentiable terms


def test_triangle_and_torque_force_vjp_match_oracle_differences():
    x, tris, mats = plate(nx=5, ny=4)
    lo, hi = tris[:, 0], tris[:, 1]
    springs = np.unique(np.sort(np.stack([lo, hi], 1), axis=1), axis=0).astype(np.int32)
    S = len(springs)
    d = x[springs[:, 1]] - x[springs[:, 0]]
    rest_dir = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    model, solver, oracle = make_pair(x, np.full(len(x), 1e-3), tris=tris, tri_materials=mats, springs=springs,
                                      spring_ke=np.full(S, 50.0, np.float32), spring_kd=np.full(S, 0.1, np.float32),
                                      spring_rest_direction=rest_dir, torque_stiffness=2.0, torque_damping=0.03)
    rng = np.random.default_rng(8)
    q = rounded(x + rng.normal(0, 1.5e-3, x.shape))
    v = rounded(rng.normal(0, 0.3, x.shape))
    g = rounded(rng.normal(0, 1.0, x.shape))
    lib = _lib.load()
    qt, vt, gt = tensor(q), tensor(v), tensor(g)  # held: the library reads them asynchronously
    qb, vb = torch.zeros(x.shape, device=DEVICE), torch.zeros(x.shape, device=DEVICE)
    _lib.check(lib.fem_force_vjp(solver._handle, qt.data_ptr(), vt.data_ptr(), None, model.gravity.data_ptr(),
                                 gt.data_ptr(), qb.data_ptr(), vb.data_ptr(), None, None,
                                 torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    qb, vb = to_np(qb), to_np(vb)

    def total(qq, vv):
        return sum(oracle.forces(qq, vv, terms=("spring", "tri")).values())

    eps = 1e-7
    for _ in range(3):
        dq, dv = rng.normal(size=x.shape), rng.normal(size=x.shape)
        want_q = np.sum(g * (total(q + eps * dq, v) - total(q - eps * dq, v))) / (2 * eps)
        want_v = np.sum(g * (total(q, v + eps * dv) - total(q, v - eps * dv))) / (2 * eps)
        np.testing.assert_allclose(np.sum(qb * dq), want_q, rtol=1e-3)
        np.testing.assert_allclose(np.sum(vb * dv), want_v, rtol=1e-3)


def test_force_vjp_refuses_contact_terms():
    x, radius, flags, v = particle_cloud(P=100)
    model, solver, _ = make_pair(x, np.full(len(x), 1e-3), radius=radius, particle_contact=(1e3, 1e2, 1e2, 0.5, 0.0),
                                 with_oracle=False)
    lib = _lib.load()
    z = torch.zeros(x.shape, device=DEVICE)
    code = lib.fem_force_vjp(solver._handle, z.data_ptr(), z.data_ptr(), None, model.gravity.data_ptr(), z.data_ptr(),
                             z.data_ptr(), z.data_ptr(), None, None, torch.cuda.current_stream().cuda_stream)
    assert code == _lib.FEM_ERR_UNSUPPORTED
