"""Shared test fixtures: the reference test suite's meshes and solver settings.

``cube`` restates ``tests/test_solver.py:176-183`` and ``tests/fem_fixture.py:17-41``
of the reference: the bundled 27-node grid (Tet4 or Hex8) scaled to a 0.1 m cube
at z = 0.3, density 100, mu = 500, lambda = 1000, damping 0, radius 0.004.
"""

from pathlib import Path

import numpy as np

from newton_solver_fem_gb300 import scenes

GOLDEN = np.load(Path(__file__).parent / "golden" / "fixture_meshes.npz")
DT = 0.002


def mesh(name):
    points = GOLDEN[f"{name}/points"].astype(np.float64)
    key = "tets" if f"{name}/tets" in GOLDEN.files else "hexes"
    return points, GOLDEN[f"{name}/{key}"].astype(np.int32)


def cube_arrays(kind="tet", density=100.0, material=(500.0, 1000.0, 0.0)):
    """Vertices, elements, masses and materials of the reference's ``cube(kind)``."""
    points, elements = mesh(f"{kind}_grid")
    x = points - points.min(axis=0)
    x *= 0.1 / np.max(np.ptp(x, axis=0))
    x += (0.0, 0.0, 0.3)
    if kind == "tet":
        mass = scenes.tet_lumped_mass(x, elements, density)
    else:
        mass = scenes.hex_lumped_mass(x, elements, density)
    mats = np.tile(np.asarray(material, np.float32), (len(elements), 1))
    return x, elements, mass, mats


def oracle_cube(kind="tet", density=100.0, gravity=(0.0, 0.0, 0.0), **options):
    from oracle import fem_oracle as O

    x, el, mass, mats = cube_arrays(kind, density)
    args = dict(dt=DT, maxiter=128, min_stretch=-1.0, gravity=gravity, radius=0.004)
    args.update(options)
    if kind == "tet":
        return O.OracleFEM(x, mass, tets=el, tet_poses=scenes.tet_poses(x, el), tet_materials=mats, **args)
    inv, det = O.hex_builder_data(x, el)
    return O.OracleFEM(x, mass, hexes=el, hex_inv_J0=inv.astype(np.float32), hex_det_J0_w=det.astype(np.float32),
                       hex_materials=mats, **args)


def one_tet():
    """Four nodes of mass 1e-3 and one tet (mu 5000, lambda 10000), ``tests/test_fixed_particles.py:31-36``."""
    x = np.array(((0, 0, 0), (0.1, 0, 0), (0, 0.1, 0), (0, 0, 0.1)), np.float64)
    tets = np.array([[0, 1, 2, 3]], np.int32)
    mats = np.array([[5000.0, 10000.0, 0.0]], np.float32)
    return x, tets, np.full(4, 1.0e-3), mats


def energy(x_rest, q, tets=None, poses=None, tet_mats=None, hexes=None, hex_mats=None):
    """Independent smooth Stable Neo-Hookean energy, restating ``tests/test_solver.py:208-229``."""
    from oracle import fem_oracle as O

    samples = []
    if tets is not None and len(tets):
        for ids, pose, material in zip(tets, poses, tet_mats):
            gradient = np.vstack((-pose.sum(axis=0), pose)).astype(np.float64)
            samples.append((ids, gradient, 1.0 / (6.0 * np.linalg.det(pose.astype(float))), material))
    if hexes is not None and len(hexes):
        inv, det = O.hex_builder_data(x_rest, hexes)
        grads = O.hex_shape_gradients(inv)
        for nodes, gs, vs, material in zip(hexes, grads, det, hex_mats):
            samples.extend((nodes, g, v, material) for g, v in zip(gs, vs))
    result = 0.0
    for ids, gradients, volume, material in samples:
        F = q[ids].T @ gradients
        ic, J = np.sum(F * F), np.linalg.det(F)
        mu, lam = float(material[0]), float(material[1])
        alpha = 1.0 + 0.75 * mu / lam
        result += volume * (0.5 * mu * (ic - 3.0) - 0.5 * mu * np.log(ic + 1.0) + 0.5 * lam * (J - alpha) ** 2)
    return result
