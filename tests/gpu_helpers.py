"""Build matching (GPU solver, CPU oracle) pairs from identical float32 inputs."""

import numpy as np
import torch

from newton_solver_fem_gb300 import SolverFEM, model_from_arrays, scenes
from oracle import fem_oracle as O

DEVICE = "cuda:0"


def rounded(a):
    return np.asarray(a, np.float32).astype(np.float64)


def make_pair(x, mass, *, tets=None, tet_materials=None, hexes=None, hex_materials=None, springs=None, spring_ke=None,
              spring_kd=None, velocity=None, radius=0.0, gravity=(0.0, 0.0, -9.81), fixed=None, dt=1.0 / 600.0,
              scene_offsets=None, solver_type="cg", preconditioner_type="block_diag", with_oracle=True, tris=None,
              tri_materials=None, flags=None, particle_contact=None, soft_contact=None, **kw):
    """Return (model, solver, oracle) over the same float32 data.

    ``particle_contact`` = (ke, kd, kf, mu, cohesion) turns on the hash-grid
    self contact; ``soft_contact`` = (ke, kd, kf, mu) sets the soft-contact
    material; ``spring_rest_direction`` / ``torque_*`` pass through to both."""
    x32 = rounded(x)
    m32 = rounded(mass)
    model = model_from_arrays(x32, m32, tets=tets, tet_materials=tet_materials, hexes=hexes,
                              hex_materials=hex_materials, springs=springs, spring_ke=spring_ke, spring_kd=spring_kd,
                              velocity=velocity, radius=radius, gravity=gravity, scene_offsets=scene_offsets,
                              tris=tris, tri_materials=tri_materials, particle_grid=particle_contact is not None,
                              device=DEVICE)
    if flags is not None:
        model.particle_flags.copy_(torch.tensor(np.asarray(flags, np.int32), device=DEVICE))
    args = dict(dt=dt, solver_type=solver_type, preconditioner_type=preconditioner_type, self_contact_ke=0.0)
    if particle_contact is not None:
        ke, kd, kf, mu, coh = particle_contact
        args.update(self_contact_ke=ke, self_contact_kd=kd)
        model.particle_kf, model.particle_mu, model.particle_cohesion = kf, mu, coh
    if soft_contact is not None:
        model.soft_contact_ke, model.soft_contact_kd, model.soft_contact_kf, model.soft_contact_mu = soft_contact
    args.update(kw)
    solver = SolverFEM(model, fixed_particle_indices=fixed, **args)
    if not with_oracle:
        return model, solver, None
    okw = dict(
        dt=dt, gravity=gravity, radius=radius, fixed=fixed,
        min_stretch=args.get("min_stretch", 0.05), max_stretch=args.get("max_stretch", 20.0),
        maxiter=args.get("linear_solver_maxiter", 50), tolerance=args.get("linear_solver_tolerance", 1e-2),
        ground_plane=args.get("ground_plane"), ground_ke=args.get("ground_ke", 1.0e5),
        ground_kd=args.get("ground_kd", 1.0e2), ground_kf=args.get("ground_kf", 1.0e3),
        ground_mu=args.get("ground_mu", 0.5), linear_damping=args.get("linear_damping", 0.0),
        preconditioner=preconditioner_type, scene_offsets=scene_offsets,
        flags=None if flags is None else np.asarray(flags, np.int32),
        spring_rest_direction=args.get("spring_rest_direction"), torque_stiffness=args.get("torque_stiffness", 0.0),
        torque_damping=args.get("torque_damping", 0.0),
        particle_contact=None if particle_contact is None else tuple(np.float32(c) for c in particle_contact),
        soft_contact=tuple(np.float32(c) for c in (model.soft_contact_ke, model.soft_contact_kd,
                                                   model.soft_contact_kf, model.soft_contact_mu)),
    )
    if tris is not None and len(tris):
        okw.update(tris=tris, tri_poses=model.tri_poses.cpu().numpy(),
                   tri_materials=np.asarray(tri_materials, np.float32))
    if tets is not None and len(tets):
        okw.update(tets=tets, tet_poses=model.tet_poses.cpu().numpy(), tet_materials=np.asarray(tet_materials,
                                                                                             np.float32))
    if hexes is not None and len(hexes):
        okw.update(hexes=hexes, hex_inv_J0=model.fem.hex_inv_J0.cpu().numpy(),
                   hex_det_J0_w=model.fem.hex_det_J0_w.cpu().numpy(),
                   hex_materials=np.asarray(hex_materials, np.float32))
    if springs is not None and len(springs):
        okw.update(springs=springs, spring_rest=model.spring_rest_length.cpu().numpy(),
                   spring_ke=np.asarray(spring_ke, np.float32), spring_kd=np.asarray(spring_kd, np.float32))
    oracle = O.OracleFEM(x32, m32, **okw)
    return model, solver, oracle


def scene_pair(scene, **kw):
    args = dict(tets=scene.tets if len(scene.tets) else None, tet_materials=scene.tet_materials,
                hexes=scene.hexes if len(scene.hexes) else None, hex_materials=scene.hex_materials,
                springs=scene.springs if len(scene.springs) else None, spring_ke=scene.spring_ke,
                spring_kd=scene.spring_kd, velocity=scene.velocity, radius=scene.radius, gravity=scene.gravity,
                fixed=scene.fixed if len(scene.fixed) else None, dt=scene.dt, scene_offsets=scene.scene_offsets,
                linear_solver_maxiter=scene.maxiter, linear_solver_tolerance=scene.tolerance)
    if scene.ground_plane is not None:
        args["ground_plane"] = scene.ground_plane
        args.update(zip(("ground_ke", "ground_kd", "ground_kf", "ground_mu"), scene.ground))
    args.update(kw)
    return make_pair(scene.x, scene.mass, **args)


def to_np(t):
    return t.detach().cpu().numpy().astype(np.float64)


def tensor(a):
    return torch.tensor(np.asarray(a, np.float32), device=DEVICE)


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def small_batch(count=6, seed=11):
    return scenes.batched_scenes(count=count, seed=seed, dims=(2, 5))


def face_triangles(x, axis, value):
    """Counter-clockwise (outward +axis) triangles over the grid nodes of the face x[:, axis] == value."""
    nodes = np.nonzero(np.isclose(x[:, axis], value))[0]
    a, b = [k for k in range(3) if k != axis]
    ua, ub = np.unique(np.round(x[nodes, a], 9)), np.unique(np.round(x[nodes, b], 9))
    grid = {(np.searchsorted(ua, round(x[n, a], 9)), np.searchsorted(ub, round(x[n, b], 9))): n for n in nodes}
    tris = []
    for i in range(len(ua) - 1):
        for j in range(len(ub) - 1):
            p00, p10, p11, p01 = grid[i, j], grid[i + 1, j], grid[i + 1, j + 1], grid[i, j + 1]
            tris += [(p00, p10, p11), (p00, p11, p01)]
    return np.asarray(tris, np.int32)


def mixed_model(seed=5):
    """A Hex8 block and a Tet4 block (Rayleigh damping) joined by springs, two supports on each, and
    membrane triangles (with drag and lift) over the hex block's top face."""
    xh, hexes, mh, massh = scenes.hex_block(2, 2, 2, 0.05, (0.0, 0.0, 0.0), 2.0e5, 0.4, 1000.0, k_damp=2.0)
    xt, tets, mt, masst = scenes.tet_block(2, 2, 2, 0.05, (0.15, 0.0, 0.0), 1.0e5, 0.45, 1000.0, k_damp=1.0)
    off = len(xh)
    x = np.concatenate([xh, xt])
    mass = np.concatenate([massh, masst])
    right_face = np.nonzero(np.isclose(xh[:, 0], 0.1))[0]
    left_face = off + np.nonzero(np.isclose(xt[:, 0], 0.15))[0]
    springs = np.stack([right_face, left_face], axis=1).astype(np.int32)
    rng = np.random.default_rng(seed)
    vel = rounded(rng.normal(0, 0.05, x.shape))
    tris = face_triangles(xh, 2, 0.1)
    tri_materials = np.tile(np.array([[30.0, 50.0, 0.03, 0.2, 0.1]], np.float32), (len(tris), 1))
    model = model_from_arrays(rounded(x), rounded(mass), tets=tets + off, tet_materials=mt, hexes=hexes,
                              hex_materials=mh, springs=springs, spring_ke=np.full(len(springs), 500.0, np.float32),
                              spring_kd=np.full(len(springs), 0.5, np.float32), velocity=vel,
                              tris=tris, tri_materials=tri_materials, gravity=(0.0, 0.0, -9.81), device=DEVICE)
    fixed = np.array([0, 1, off + len(xt) - 1, off + len(xt) - 2], np.int32)
    return model, fixed, rng
