"""Pin the CPU oracle to the reference's own known-answer tests (no GPU needed).

Each test restates one hot-path check of the reference's test suite on the same
fixture meshes (read from ``tests/golden/fixture_meshes.npz``) with the same
tolerances; the reference file:line is in each docstring.
"""

import numpy as np
import pytest
from fixtures import DT, cube_arrays, energy, one_tet, oracle_cube

from newton_solver_fem_gb300 import scenes
from oracle import fem_oracle as O


def test_hex_box_quadrature_and_one_step_fall():
    """Hex 2x3x4 box: det_J0_w = 3, inv_J0 = diag(1, 2/3, 1/2), dv_z = -0.00981 (tests/test_reference_builder.py:35-54)."""
    nodes = np.asarray([(0, 0, 0), (2, 0, 0), (2, 3, 0), (0, 3, 0), (0, 0, 4), (2, 0, 4), (2, 3, 4), (0, 3, 4)], float)
    inv, det = O.hex_builder_data(nodes, np.arange(8).reshape(1, 8))
    np.testing.assert_allclose(det, 3.0)
    np.testing.assert_allclose(inv.astype(np.float32), np.broadcast_to(np.diag([1.0, 2 / 3, 0.5]), (1, 8, 3, 3)),
                               atol=2e-7)
    solver = O.OracleFEM(nodes, np.full(8, 3.0), hexes=np.arange(8).reshape(1, 8), hex_inv_J0=inv.astype(np.float32),
                         hex_det_J0_w=det.astype(np.float32), hex_materials=np.array([[10, 20, 0]], np.float32),
                         dt=0.001, gravity=(0, 0, -9.81))
    _, v, _ = solver.step(nodes, np.zeros((8, 3)), 0.001)
    np.testing.assert_allclose(v[:, 2], -0.00981, atol=1e-7)


def test_grid_volume_and_mass():
    """Hex grid sums to 0.1^3 and mass 100*0.1^3 (tests/test_solver.py:505-512)."""
    x, el, mass, _ = cube_arrays("hex")
    _, det = O.hex_builder_data(x, el)
    assert abs(float(det.astype(np.float32).sum()) - 0.1**3) < 1e-8
    assert abs(float(mass.sum()) - 100 * 0.1**3) < 1e-6


@pytest.mark.parametrize("kind", ["tet", "hex"])
def test_rigid_motion_symmetry_and_spd(kind):
    """Rest forces vanish under rigid motion; A symmetric and SPD (tests/test_solver.py:336-348)."""
    rotation = np.array([[0.8, -0.6, 0.0], [0.6, 0.8, 0.0], [0.0, 0.0, 1.0]])
    solver = oracle_cube(kind)
    q = solver.rest @ rotation.T + [0.1, 0.2, -0.15]
    f = solver.forces(q, np.zeros_like(q), terms=("tet", "hex"))
    np.testing.assert_allclose(f["tet"] + f["hex"], 0, atol=3e-4)
    A = solver.dense()
    np.testing.assert_allclose(A, A.T, atol=2e-8)
    assert np.linalg.eigvalsh(A).min() > 0


@pytest.mark.parametrize("kind", ["tet", "hex"])
def test_force_is_energy_gradient(kind):
    """f = -grad(energy) by central differences, sum f = 0 (tests/test_solver.py:350-368)."""
    rng = np.random.default_rng(7)
    solver = oracle_cube(kind)
    x, el, _, mats = cube_arrays(kind)
    q = x.copy()
    q[:, 0] *= 1.08
    q[:, 1] += 0.04 * q[:, 2]
    f = solver.forces(q, np.zeros_like(q), terms=("tet", "hex"))
    force = f["tet"] + f["hex"]
    direction = rng.normal(size=q.shape)
    direction /= np.linalg.norm(direction)
    if kind == "tet":
        kw = dict(tets=el, poses=scenes.tet_poses(x, el), tet_mats=mats)
    else:
        kw = dict(hexes=el, hex_mats=mats)
    for eps in (1e-4, 5e-5):
        diff = (energy(x, q + eps * direction, **kw) - energy(x, q - eps * direction, **kw)) / (2 * eps)
        np.testing.assert_allclose(float(-(force * direction).sum()), diff, rtol=0.001, atol=3e-5)
    np.testing.assert_allclose(force.sum(axis=0), 0, atol=2e-5)


def test_step_matches_dense_solve():
    """One step equals the dense solve of A dv = h f - (A - M) v (tests/test_solver.py:232-262)."""
    solver = oracle_cube("tet", tolerance=1e-12)
    q = solver.rest.copy()
    q[-1, 2] -= 0.001
    velocity = np.random.default_rng(2).normal(0, 0.03, q.shape).astype(np.float32).astype(np.float64)
    force = np.zeros_like(q)
    force[-1] = (0.1, 0.05, -0.2)
    mass = np.repeat(solver.mass, 3)
    A = solver.dense()
    elastic = solver.forces(q, velocity, terms=("tet",))["tet"]
    rhs = DT * (force + elastic).ravel() - A @ velocity.ravel() + mass * velocity.ravel()
    increment = np.linalg.solve(A, rhs).reshape(q.shape)
    q_out, v_out, _ = solver.step(q, velocity, DT, external=force)
    np.testing.assert_allclose(v_out, velocity + increment, rtol=3e-4, atol=3e-6)
    np.testing.assert_allclose(q_out, q + DT * (velocity + increment), rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("density", [0.1, 1000.0])
def test_freefall_across_mass_scales(density):
    """Zero RHS keeps the state; gravity gives dv_z = -g h (tests/test_solver.py:440-450).

    The reference's ``make_solver`` defaults to ``differentiable=True``, whose checked solve uses tol 1e-8.
    """
    solver = oracle_cube("tet", density=density, tolerance=1e-8)
    q0 = solver.rest.copy()
    q, _, _ = solver.step(q0, np.zeros_like(q0), DT)
    np.testing.assert_allclose(q, q0, atol=2e-7)
    solver.gravity = np.array([0.0, 0.0, -9.81])
    _, v, _ = solver.step(q0, np.zeros_like(q0), DT)
    np.testing.assert_allclose(v[:, 2], -DT * 9.81, atol=2e-5)


@pytest.mark.parametrize("mass", [1e-25, 1e-18, 1e-14, 1.0])
def test_tiny_mass_falls_and_zero_rhs_clears_warm_start(mass):
    """RHS normalisation keeps tiny masses falling; b = 0 clears dv (tests/test_reference_block_preconditioner.py:71-91)."""
    dt = 1 / 240
    solver = O.OracleFEM(np.array([[0.0, 0.0, 1.0]]), np.array([mass]), gravity=(0, 0, -9.81), dt=dt, maxiter=8)
    q, v = solver.rest.copy(), np.zeros((1, 3))
    for step in range(1, 4):
        q, v, rhs = solver.step(q, v, dt)
        np.testing.assert_allclose(v[0], (0, 0, -step * 9.81 * dt), atol=1e-7)
        np.testing.assert_allclose(solver.dv[0], (0, 0, -9.81 * dt), atol=1e-7)
        np.testing.assert_allclose(rhs[0], (0, 0, -mass * 9.81 * dt), rtol=3e-7, atol=0)
    solver.gravity = np.zeros(3)
    q2, v2, _ = solver.step(q, v, dt)
    np.testing.assert_allclose(v2, v, atol=1e-7)
    np.testing.assert_array_equal(solver.dv, np.zeros((1, 3)))


def test_dirichlet_matches_reduced_system():
    """Fixed nodes: the free block solves the reduced dense system (tests/test_fixed_particles.py:50-79)."""
    x, tets, mass, mats = one_tet()
    solver = O.OracleFEM(x, mass, tets=tets, tet_poses=scenes.tet_poses(x, tets), tet_materials=mats, gravity=(0, 0, 0),
                         dt=DT, fixed=[0, 1], maxiter=64, tolerance=1e-12)
    q = x.copy()
    q[2] += (0.002, 0.001, -0.001)
    velocity = np.array(((0, 0, 0), (0, 0, 0), (0.02, -0.03, 0.01), (-0.01, 0.01, 0.02)), np.float64)
    external = np.array(((20, 30, 40), (10, -30, 60), (0.02, 0.04, 0.03), (-0.01, 0.03, 0.02)), np.float64)
    for refresh in (False, True, True):
        if refresh:
            q = solver.refresh_tangent(q)
        A = solver.dense()
        elastic = solver.forces(q, velocity, terms=("tet",))["tet"]
        m = np.repeat(solver.mass, 3)
        rhs = DT * (elastic + external).ravel() - (A - np.diag(m)) @ velocity.ravel()
        expected = np.zeros(12)
        expected[6:] = np.linalg.solve(A[6:, 6:], rhs[6:])
        q_out, v_out, _ = solver.step(q, velocity, DT, external=external)
        np.testing.assert_allclose(solver.dv.ravel(), expected, rtol=3e-4, atol=2e-6)
        np.testing.assert_array_equal(q_out[:2], x[:2])
        np.testing.assert_array_equal(v_out[:2], np.zeros((2, 3)))
        q, velocity = q_out, v_out


def test_block_inverse_scale_invariance_and_fallback():
    """Scale-normalised inverse over 1e-20..1e20, singular fallback (tests/test_reference_block_preconditioner.py:48-69)."""
    base = np.asarray(((4, 0.7, -0.3), (0.7, 2, 0.4), (-0.3, 0.4, 1)), dtype=np.float64)
    scales = np.power(10.0, np.arange(-20, 21, dtype=float))
    blocks = (scales[:, None, None] * base).astype(np.float32)
    expected = np.linalg.inv(blocks.astype(np.float64))
    inverse = O.inverse_diagonal_block(blocks, dtype=np.float32)
    assert np.isfinite(inverse).all()
    np.testing.assert_allclose(inverse, expected, rtol=6e-7, atol=0)
    singular = (scales[:, None, None] * np.diag((1, 0, 2))).astype(np.float32)
    want = np.zeros_like(singular)
    want[:, 0, 0] = 1 / singular[:, 0, 0]
    want[:, 1, 1] = 1
    want[:, 2, 2] = 1 / singular[:, 2, 2]
    np.testing.assert_allclose(O.inverse_diagonal_block(singular, dtype=np.float32), want, rtol=2e-7, atol=0)


def test_tolerance_semantics():
    """True relative residual < 0.0101 at tol 1e-2 and < 2e-5 at 1e-5 with more iterations (tests/test_solver.py:281-316)."""
    external = np.random.default_rng(13).normal(0, 0.03, (27, 3)).astype(np.float32).astype(np.float64)
    residuals, iterations = [], []
    for tol in (1e-2, 1e-5):
        solver = oracle_cube("tet", tolerance=tol)
        q0 = solver.rest.copy()
        _, _, rhs = solver.step(q0, np.zeros_like(q0), DT, external=external)
        A = solver.dense()
        residuals.append(np.linalg.norm(A @ solver.dv.ravel() - rhs.ravel()) / np.linalg.norm(rhs))
        iterations.append(solver.last_iterations[0])
    assert residuals[0] < 0.0101
    assert residuals[1] < 2e-5
    assert iterations[1] > iterations[0]


def test_unique_edge_springs():
    """Two tets sharing a face give 9 unique edges (tests/test_reference_builder.py:15-33)."""
    x = np.array([(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 0, -1)], float)
    tets = np.array([[0, 1, 2, 3], [0, 2, 1, 4]], np.int32)
    assert len(scenes.unique_edges(x, tets)) == 9


def test_external_force_derivative_is_half_dt():
    """A free 2 kg particle has d v_x / d f_ext = h/2 (tests/test_solver.py:452-464), by linearity."""
    solver = O.OracleFEM(np.array([[0.0, 0.0, 1.0]]), np.array([2.0]), gravity=(0, 0, 0), dt=DT, maxiter=128,
                         tolerance=1e-12)
    eps = 1e-3
    _, vp, _ = solver.step(solver.rest, np.zeros((1, 3)), DT, external=np.array([[eps, 0, 0]]))
    _, vm, _ = solver.step(solver.rest, np.zeros((1, 3)), DT, external=np.array([[-eps, 0, 0]]))
    np.testing.assert_allclose((vp[0, 0] - vm[0, 0]) / (2 * eps), DT / 2, atol=1e-8)


def test_synthetic_config_sizes():
    """Workload sizes: Tet4 8x2x2 -> 81 nodes / 192 tets / nnzb 769; 16x4x4 -> 425 / 1536 / 4921."""
    c1 = scenes.tet_cantilever()
    assert (c1.particle_count, len(c1.tets), len(c1.fixed)) == (81, 192, 9)
    assert np.all(scenes.tet_volumes(c1.x, c1.tets) > 0)
    r, c, v = O.constant_triplets(c1.mass, np.zeros((0, 2), np.int64), np.zeros(0), np.zeros(0), c1.dt)
    rt, ct, vt = O.tet_tangent(c1.x, c1.tets, scenes.tet_poses(c1.x, c1.tets), c1.tet_materials, 0.05, 20.0, c1.dt)
    offsets, _, _ = O.assemble_bsr(np.concatenate([r, rt]), np.concatenate([c, ct]), np.concatenate([v, vt]), 81)
    assert offsets[-1] == 769
    c4 = scenes.tet_beam()
    assert (c4.particle_count, len(c4.tets)) == (425, 1536)
    hx = scenes.hex_cells(2, 2, 2)
    xg = scenes.grid_nodes(2, 2, 2, 0.05)
    assert hx.shape == (8, 8)
    _, det = O.hex_builder_data(xg, hx)
    np.testing.assert_allclose(det.sum(), 0.1**3)


# ---------------------------------------------------------------- triangles, torque springs, contacts


def _membrane():
    from newton_solver_fem_gb300.builder import triangle_rest_data

    g = np.stack(np.meshgrid(np.arange(4) * 0.02, np.arange(3) * 0.02, indexing="ij"), -1).reshape(-1, 2)
    x = np.column_stack([g, np.full(len(g), 0.1)])
    tris = []
    for i in range(3):
        for j in range(2):
            a, b, c, d = 3 * i + j, 3 * (i + 1) + j, 3 * (i + 1) + j + 1, 3 * i + j + 1
            tris += [(a, b, c), (a, c, d)]
    tris = np.asarray(tris)
    poses, area = triangle_rest_data(x, tris)
    mats = np.tile([[30.0, 50.0, 0.0, 0.0, 0.0]], (len(tris), 1))
    return x, tris, poses, area, mats


def test_triangle_pose_is_the_inverse_rest_edge_matrix_in_the_triangle_frame():
    """Newton's triangle pose: inv([[e1.x10, e1.x20], [e2.x10, e2.x20]]) with e1 along x10 and area det/2."""
    from newton_solver_fem_gb300.builder import triangle_rest_data

    x = np.array([[0.0, 0.0, 0.0], [0.1, 0.0, 0.0], [0.0, 0.1, 0.0], [0.1, 0.1, 0.0]])
    poses, area = triangle_rest_data(x, [[0, 1, 2], [0, 1, 3]])
    np.testing.assert_allclose(poses[0], np.diag([10.0, 10.0]), atol=1e-12)
    np.testing.assert_allclose(poses[1], [[10.0, -10.0], [0.0, 10.0]], atol=1e-12)
    np.testing.assert_allclose(area, [0.005, 0.005])
    # the kernels' rest area 1 / (2 det pose) is the same area
    np.testing.assert_allclose(1.0 / (2.0 * np.linalg.det(poses)), area)


def test_triangle_membrane_force_is_the_energy_gradient_and_conserves_momentum():
    """f = -dE/dx for E = mu' (I_C/2 - ln I_C) + lambda' c^2 / 2 per triangle (rest-area scaled), zero at rest."""
    x, tris, poses, area, mats = _membrane()
    rng = np.random.default_rng(0)
    np.testing.assert_allclose(O.triangle_forces(x, np.zeros_like(x), tris, poses, mats), 0.0, atol=1e-12)
    q = x + rng.normal(0, 2e-3, x.shape)

    def energy_of(p):
        e = 0.0
        for t, Dm, m, a0 in zip(tris, poses, mats, area):
            F = np.column_stack([p[t[1]] - p[t[0]], p[t[2]] - p[t[0]]]) @ Dm
            Ic = np.sum(F * F)
            c = 0.5 * np.linalg.norm(np.cross(p[t[1]] - p[t[0]], p[t[2]] - p[t[0]])) / a0 - 1.0
            e += a0 * m[0] * (0.5 * Ic - np.log(Ic)) + 0.5 * a0 * m[1] * c * c
        return e

    f = O.triangle_forces(q, np.zeros_like(q), tris, poses, mats)
    eps = 1e-7
    for _ in range(3):
        d = rng.normal(size=q.shape)
        de = (energy_of(q + eps * d) - energy_of(q - eps * d)) / (2 * eps)
        np.testing.assert_allclose(np.sum(f * d), -de, rtol=1e-5)
    np.testing.assert_allclose(f.sum(0), 0.0, atol=1e-10)
    # drag and lift act along the mean velocity and the normal only
    mats_air = mats.copy()
    mats_air[:, 3:] = (0.4, 0.3)
    v = np.tile([[0.0, 0.0, 1.0]], (len(x), 1))
    f_air = O.triangle_forces(x, v, tris, poses, mats_air)
    np.testing.assert_allclose(f_air[:, :2], 0.0, atol=1e-12)
    assert f_air[:, 2].min() < 0.0  # the 0.3333 mean-velocity drag and the lift oppose upward motion at corner 0


def test_triangle_lumped_blocks():
    """h^2 (mu + lambda) A_rest / 3 I on each vertex, zero for a degenerate triangle (kernels.py:963-1012)."""
    x, tris, poses, area, mats = _membrane()
    rows, cols, vals = O.triangle_triplets(tris, poses, mats, 0.01)
    np.testing.assert_array_equal(rows, tris.reshape(-1))
    np.testing.assert_allclose(vals[0], 1e-4 * (30.0 + 50.0) * area[0] / 3.0 * np.eye(3))
    _, _, degenerate = O.triangle_triplets(tris[:1], np.zeros((1, 2, 2)), mats[:1], 0.01)
    assert not degenerate.any()


def test_spring_torque_vanishes_at_rest_and_conserves_momentum():
    rng = np.random.default_rng(1)
    x = np.cumsum(rng.normal(0, 0.02, (6, 3)) + (0.03, 0, 0), axis=0)
    springs = np.array([(0, 1), (1, 2), (2, 3), (3, 4), (4, 5)])
    d = x[springs[:, 1]] - x[springs[:, 0]]
    rest = d / np.linalg.norm(d, axis=1, keepdims=True)
    np.testing.assert_allclose(O.spring_torque_forces(x, np.zeros_like(x), springs, rest, 2.0, 0.1), 0.0, atol=1e-12)
    q = x + rng.normal(0, 3e-3, x.shape)
    v = rng.normal(0, 0.2, x.shape)
    f = O.spring_torque_forces(q, v, springs, rest, 2.0, 0.1)
    assert np.abs(f).max() > 0
    np.testing.assert_allclose(f.sum(0), 0.0, atol=1e-12)
    # transverse: no component along each spring (a single spring isolates its own force)
    one = O.spring_torque_forces(q, v, springs[:1], rest[:1], 2.0, 0.1)
    axis = q[0] - q[1]
    assert abs(np.dot(one[1], axis)) < 1e-10 * np.linalg.norm(one[1]) * np.linalg.norm(axis)


def test_particle_contact_pairs_are_equal_and_opposite():
    rng = np.random.default_rng(2)
    x = rng.uniform(0, 0.1, (60, 3))
    radius = rng.uniform(0.005, 0.01, 60)
    v = rng.normal(0, 0.3, (60, 3))
    flags = np.ones(60, np.int32)
    f = O.particle_contact_forces(x, v, radius, flags, 1e3, 1e2, 1e2, 0.5, 0.0)
    assert (np.abs(f).sum(1) > 0).sum() > 10
    np.testing.assert_allclose(f.sum(0), 0.0, atol=1e-9 * np.abs(f).max())
    # two particles: penalty along the line of centres, err = d - r_i - r_j
    two = O.particle_contact_forces(np.array([[0, 0, 0], [0.015, 0, 0]]), np.zeros((2, 3)), np.array([0.01, 0.01]),
                                    np.ones(2, np.int32), 1e3, 1e2, 1e2, 0.5, 0.0)
    np.testing.assert_allclose(two, [[-5.0, 0, 0], [5.0, 0, 0]])


def test_soft_contact_known_answer():
    """One penetrating contact: fn = ke pen - kd min(vn, 0); friction capped by mu max(fn, 0) (kernels.py:1198-1261)."""
    x = np.array([[0.0, 0.0, 0.009]])
    v = np.array([[0.3, 0.0, -0.2]])
    f = O.soft_contact_forces(x, v, np.array([0.01]), 1, np.array([0]), np.zeros((1, 3)), np.zeros((1, 3)),
                              np.array([[0.0, 0.0, 1.0]]), 1e3, 10.0, 1e3, 0.5)
    fn = 1e3 * 0.001 + 10.0 * 0.2
    np.testing.assert_allclose(f, [[-min(1e3 * 0.3, 0.5 * fn), 0.0, fn]])
    none = O.soft_contact_forces(x + (0, 0, 0.01), v, np.array([0.01]), 1, np.array([0]), np.zeros((1, 3)),
                                 np.zeros((1, 3)), np.array([[0.0, 0.0, 1.0]]), 1e3, 10.0, 1e3, 0.5)
    assert not none.any()


# ---------------------------------------------------------------- surface contacts


def _tet_block_surface(x, tets):
    """Boundary faces of a tet mesh, oriented outward."""
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
    return np.asarray(out, np.int64)


def test_closest_point_on_triangle_regions():
    a, b, c = np.array([[0.0, 0, 0]]), np.array([[1.0, 0, 0]]), np.array([[0.0, 1, 0]])
    for p, want, feat in (((0.2, 0.2, 0.5), (0.2, 0.2, 0.0), 0), ((-1.0, -1.0, 0.3), (0, 0, 0), 4),
                          ((2.0, -0.5, 0.0), (1, 0, 0), 5), ((0.5, -1.0, 0.0), (0.5, 0, 0), 1),
                          ((1.0, 1.0, 0.0), (0.5, 0.5, 0), 2), ((-1.0, 0.5, 0.0), (0, 0.5, 0), 3)):
        pts, f = O.closest_on_triangles(np.asarray(p, float), a, b, c)
        np.testing.assert_allclose(pts[0], want, atol=1e-12)
        assert f[0] == feat


def test_pseudonormal_sign_separates_inside_from_outside_a_closed_surface():
    """Angle-weighted pseudonormals give the exact inside/outside sign of a closed mesh (Baerentzen-Aanaes)."""
    x, tets, _, _ = scenes.tet_block(2, 2, 2, 0.5, (0.0, 0.0, 0.0), 1e5, 0.4, 1000.0)
    tris = _tet_block_surface(x, tets)
    fn, vn, en = O.surface_pseudonormals(x, tris)
    rng = np.random.default_rng(0)
    for p in rng.uniform(-0.5, 1.5, (200, 3)):
        pts, feat = O.closest_on_triangles(p, x[tris[:, 0]], x[tris[:, 1]], x[tris[:, 2]])
        t = int(np.argmin(np.sum((p - pts) ** 2, 1)))
        ft = int(feat[t])
        pn = fn[t] if ft == 0 else (en[t, ft - 1] if ft <= 3 else vn[int(tris[t, ft - 4])])
        inside = bool(np.all((p > 0) & (p < 1)))
        assert (np.dot(p - pts[t], pn) < 0) == inside


def test_surface_force_pushes_a_penetrating_vertex_out_of_the_other_body():
    xa, ta, _, _ = scenes.tet_block(1, 1, 1, 0.1, (0.0, 0.0, 0.0), 1e5, 0.4, 1000.0)
    xb, tb, _, _ = scenes.tet_block(1, 1, 1, 0.1, (0.09, 0.02, 0.03), 1e5, 0.4, 1000.0)
    x = np.concatenate([xa, xb])
    bodies = [(0, len(xa), _tet_block_surface(xa, ta)), (len(xa), len(xb), _tet_block_surface(xb, tb))]
    radius = np.full(len(x), 0.004)
    f = O.surface_contact_forces(x, np.zeros_like(x), radius, np.ones(len(x), np.int32), bodies, x, x, 1e3, 1e2)
    # corner (0.1, 0.1, 0.1) of A lies 1 cm inside B along x: pushed toward -x with ke (0.01 + r)
    k = int(np.argmin(np.linalg.norm(xa - (0.1, 0.1, 0.1), axis=1)))
    np.testing.assert_allclose(f[k], (-1e3 * (0.01 + 0.004), 0.0, 0.0), atol=1e-9)
    far = int(np.argmin(np.linalg.norm(xa - (0.0, 0.0, 0.0), axis=1)))
    assert not f[far].any()
