"""Minimal Newton-style model containers and the Hex8-aware FEM builder.

The reference builds its input with Newton 1.7's ``ModelBuilder`` plus the
package's ``FEMBuilder`` extension (``builder.py:22-135``) and reads the
finalised ``Model`` / ``State`` / ``Control`` objects.  Newton is not part of
this project, so this module provides the subset of that contract the solver
hot path consumes, with PyTorch tensors on a CUDA device as storage:

* ``Model``: particle_q/qd/mass/inv_mass/radius/flags, tet_indices/poses/
  materials/activations, tri_indices/poses/materials, spring_indices/
  rest_length/stiffness/damping, gravity, ``fem`` (``LinearFEMData`` with the
  Hex8 Gauss data), the particle-contact and soft-contact coefficients,
  ``particle_grid`` and optional ``scene_offsets`` for independent batched
  scenes.
* ``State``: particle_q, particle_qd, particle_f.  ``Control``: tet_activations.
* ``Contacts``: the soft-rigid contact list (``soft_contact_*``) a collision
  pipeline produces.

Conventions follow Newton's: a tet pose is the inverse of the rest edge matrix
``[x1-x0, x2-x0, x3-x0]`` (columns) and non-positive tets are rejected; a
triangle pose is the inverse of the 2x2 rest edge matrix in the triangle's own
orthonormal frame (e1 along x1-x0, e2 = n x e1) and degenerate triangles are
rejected; Hex8 ``inv_J0`` / ``|det J0|`` are computed in float64 per Gauss
point and stored as float32 (``builder.py:95-135``).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

PARTICLE_FLAG_ACTIVE = 1

_HEX_SIGNS = np.asarray(
    [[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]],
    dtype=np.float64,
)


def hex_gauss_data(rest: np.ndarray, indices: np.ndarray):
    """Per-Gauss-point ``inv_J0`` [H,8,3,3] and ``|det J0|`` [H,8] in float64 (``builder.py:95-135``)."""
    indices = np.asarray(indices, dtype=np.int64).reshape(-1, 8)
    if len(indices) == 0:
        return np.zeros((0, 8, 3, 3)), np.zeros((0, 8))
    gp = _HEX_SIGNS / np.sqrt(3.0)
    deriv = np.empty((8, 8, 3))
    for g in range(8):
        xi, eta, zeta = gp[g]
        xa, ya, za = _HEX_SIGNS[:, 0], _HEX_SIGNS[:, 1], _HEX_SIGNS[:, 2]
        deriv[g, :, 0] = xa * (1 + ya * eta) * (1 + za * zeta) * 0.125
        deriv[g, :, 1] = (1 + xa * xi) * ya * (1 + za * zeta) * 0.125
        deriv[g, :, 2] = (1 + xa * xi) * (1 + ya * eta) * za * 0.125
    J = np.einsum("hai,gaj->hgij", np.asarray(rest, np.float64)[indices], deriv)
    det = np.linalg.det(J)
    bad = np.argwhere(det <= 1.0e-12)
    if len(bad):
        e, p = bad[0]
        raise ValueError(f"Degenerate or inverted Hex8 {e}, Gauss point {p}: {det[e, p]}")
    return np.linalg.inv(J), np.abs(det)


@dataclass
class LinearFEMData:
    """Hex8 reference geometry and materials stored under ``model.fem`` (``builder.py:12-20``)."""

    hex_count: int
    hex_indices: torch.Tensor
    hex_materials: torch.Tensor
    hex_inv_J0: torch.Tensor
    hex_det_J0_w: torch.Tensor


class State:
    """Particle state: positions, velocities and the force workspace."""

    def __init__(self, q: torch.Tensor, qd: torch.Tensor, requires_grad: bool = False):
        self.particle_q = q.clone()
        self.particle_qd = qd.clone()
        self.particle_f = torch.zeros_like(q)
        if requires_grad:
            self.particle_q.requires_grad_(True)
            self.particle_qd.requires_grad_(True)

    def clear_forces(self):
        self.particle_f.zero_()


class Control:
    """Per-step controls: Newton's per-tet activations."""

    def __init__(self, tet_activations: torch.Tensor):
        self.tet_activations = tet_activations


def triangle_rest_data(x: np.ndarray, tris: np.ndarray):
    """Rest pose ``inv(D)`` and area ``det(D)/2`` of triangles, D = [[e1.x10, e1.x20], [e2.x10, e2.x20]]
    in the frame e1 = x10/|x10|, e2 = n x e1 (n the unit normal), in float64."""
    tris = np.asarray(tris, np.int64).reshape(-1, 3)
    x = np.asarray(x, np.float64)
    x10 = x[tris[:, 1]] - x[tris[:, 0]]
    x20 = x[tris[:, 2]] - x[tris[:, 0]]
    n = np.cross(x10, x20)
    nn = np.linalg.norm(n, axis=1, keepdims=True)
    n = n / np.where(nn > 0, nn, 1.0)
    e1 = x10 / np.maximum(np.linalg.norm(x10, axis=1, keepdims=True), 1e-300)
    e2 = np.cross(n, e1)
    e2 = e2 / np.maximum(np.linalg.norm(e2, axis=1, keepdims=True), 1e-300)
    D = np.stack([np.stack([np.sum(e1 * x10, 1), np.sum(e1 * x20, 1)], 1),
                  np.stack([np.sum(e2 * x10, 1), np.sum(e2 * x20, 1)], 1)], 1)
    area = np.linalg.det(D) / 2.0 if len(D) else np.zeros(0)
    poses = np.zeros_like(D)
    ok = area > 0.0
    if ok.any():
        poses[ok] = np.linalg.inv(D[ok])
    return poses, area


class HashGrid:
    """Marks a model as carrying a particle hash grid (Newton ``wp.HashGrid(dim_x, dim_y, dim_z)``).

    The solver builds its own wrapped-bucket grid on the device from the
    particle positions at every force evaluation; the dimensions here are
    informational."""

    def __init__(self, dim_x: int = 128, dim_y: int = 128, dim_z: int = 128):
        self.dims = (int(dim_x), int(dim_y), int(dim_z))


class Contacts:
    """Soft-rigid contact list in the layout of Newton's ``Contacts.soft_contact_*``.

    ``soft_contact_count`` is a device int32 tensor of shape [1] (read on the
    device); the per-contact arrays have ``soft_contact_max`` entries: particle
    [max] int32, body_pos / body_vel / normal [max, 3] float32 (world space)."""

    def __init__(self, soft_contact_max: int, device="cuda"):
        dev = torch.device(device)
        self.soft_contact_max = int(soft_contact_max)
        self.soft_contact_count = torch.zeros(1, dtype=torch.int32, device=dev)
        self.soft_contact_particle = torch.full((self.soft_contact_max,), -1, dtype=torch.int32, device=dev)
        self.soft_contact_body_pos = torch.zeros((self.soft_contact_max, 3), dtype=torch.float32, device=dev)
        self.soft_contact_body_vel = torch.zeros((self.soft_contact_max, 3), dtype=torch.float32, device=dev)
        self.soft_contact_normal = torch.zeros((self.soft_contact_max, 3), dtype=torch.float32, device=dev)


class Model:
    """Finalised, device-resident model (the subset of Newton's ``Model`` the solver reads).

    Contact coefficients default to particle ke 1e3, kd 1e2, kf 1e2, mu 0.5,
    cohesion 0 and soft-contact ke 1e3, kd 10, kf 1e3, mu 0.5; SolverFEM sets
    ``particle_ke`` / ``particle_kd`` from ``self_contact_ke`` / ``self_contact_kd``."""

    def __init__(self, device: torch.device):
        self.device = torch.device(device)
        self.requires_grad = False
        self.tri_indices = torch.zeros((0, 3), dtype=torch.int32, device=self.device)
        self.tri_poses = torch.zeros((0, 2, 2), dtype=torch.float32, device=self.device)
        self.tri_materials = torch.zeros((0, 5), dtype=torch.float32, device=self.device)
        self.tri_areas = torch.zeros(0, dtype=torch.float32, device=self.device)
        self.particle_grid = None
        self.particle_ke = 1.0e3
        self.particle_kd = 1.0e2
        self.particle_kf = 1.0e2
        self.particle_mu = 0.5
        self.particle_cohesion = 0.0
        self.soft_contact_ke = 1.0e3
        self.soft_contact_kd = 10.0
        self.soft_contact_kf = 1.0e3
        self.soft_contact_mu = 0.5

    @property
    def particle_count(self) -> int:
        return int(self.particle_q.shape[0])

    @property
    def tet_count(self) -> int:
        return int(self.tet_indices.shape[0])

    @property
    def spring_count(self) -> int:
        return int(self.spring_indices.shape[0] // 2)

    @property
    def tri_count(self) -> int:
        return int(self.tri_indices.shape[0])

    @property
    def particle_max_radius(self) -> float:
        return float(self.particle_radius.max()) if self.particle_count else 0.0

    @property
    def scene_count(self) -> int:
        return 1 if self.scene_offsets is None else len(self.scene_offsets) - 1

    def state(self, requires_grad: bool | None = None) -> State:
        return State(self.particle_q, self.particle_qd, bool(requires_grad))

    def control(self) -> Control:
        return Control(self.tet_activations)

    def set_gravity(self, gravity) -> None:
        """Update gravity in place; solver launches (and captured graphs) read it live."""
        self.gravity.copy_(torch.as_tensor(gravity, dtype=torch.float32))


class FEMBuilder:
    """Builder for Tet4/Hex8 soft bodies with Newton's public ``ModelBuilder`` calls.

    Add particles, then connectivity with global indices; masses are the
    caller's responsibility.  ``begin_scene()`` starts an independent scene for
    batched solves (elements may not couple scenes).
    """

    default_particle_radius = 0.1
    default_tet_k_mu = 1.0e3
    default_tet_k_lambda = 1.0e3
    default_tet_k_damp = 0.0
    default_tri_ke = 100.0
    default_tri_ka = 100.0
    default_tri_kd = 10.0
    default_tri_drag = 0.0
    default_tri_lift = 0.0

    def __init__(self, gravity=(0.0, 0.0, -9.81), up_axis: str = "Z"):
        self.gravity = tuple(float(g) for g in gravity)
        self.particle_q: list = []
        self.particle_qd: list = []
        self.particle_mass: list = []
        self.particle_radius: list = []
        self.particle_flags: list = []
        self.tet_indices: list = []
        self.tet_poses: list = []
        self.tet_materials: list = []
        self.tet_activations: list = []
        self.tri_indices: list = []
        self.tri_materials: list = []
        self.spring_indices: list = []
        self.spring_rest_length: list = []
        self.spring_stiffness: list = []
        self.spring_damping: list = []
        self.fem_hex_indices: list = []
        self.fem_hex_materials: list = []
        self.scene_starts: list = []

    # ---- counts
    @property
    def particle_count(self) -> int:
        return len(self.particle_q)

    @property
    def tet_count(self) -> int:
        return len(self.tet_indices)

    @property
    def spring_count(self) -> int:
        return len(self.spring_stiffness)

    # ---- particles
    def add_particle(self, pos, vel=(0.0, 0.0, 0.0), mass=1.0, radius=None, flags=PARTICLE_FLAG_ACTIVE) -> int:
        self.particle_q.append(tuple(float(v) for v in pos))
        self.particle_qd.append(tuple(float(v) for v in vel))
        self.particle_mass.append(float(mass))
        self.particle_radius.append(self.default_particle_radius if radius is None else float(radius))
        self.particle_flags.append(int(flags))
        return len(self.particle_q) - 1

    def add_particles(self, pos, vel, mass, radius=None) -> None:
        pos = np.asarray(pos, np.float64).reshape(-1, 3)
        vel = np.asarray(vel, np.float64).reshape(-1, 3)
        mass = np.broadcast_to(np.asarray(mass, np.float64), (len(pos),))
        radius = [None] * len(pos) if radius is None else np.broadcast_to(np.asarray(radius, np.float64), (len(pos),))
        for p, v, m, r in zip(pos, vel, mass, radius):
            self.add_particle(p, v, m, r)

    def begin_scene(self) -> None:
        """Start a new independent scene at the current particle count."""
        if not self.scene_starts or self.scene_starts[-1] != self.particle_count:
            self.scene_starts.append(self.particle_count)

    # ---- elements
    def add_tetrahedron(self, i, j, k, l, k_mu=None, k_lambda=None, k_damp=None) -> float:
        """Add a Tet4 with pose inv([x1-x0, x2-x0, x3-x0]); non-positive tets are skipped (returns volume)."""
        k_mu = self.default_tet_k_mu if k_mu is None else k_mu
        k_lambda = self.default_tet_k_lambda if k_lambda is None else k_lambda
        k_damp = self.default_tet_k_damp if k_damp is None else k_damp
        p = np.asarray([self.particle_q[n] for n in (i, j, k, l)], np.float64)
        Dm = (p[1:] - p[0]).T
        volume = float(np.linalg.det(Dm)) / 6.0
        if volume <= 0.0:
            return volume
        self.tet_indices.append((int(i), int(j), int(k), int(l)))
        self.tet_poses.append(np.linalg.inv(Dm).astype(np.float32))
        self.tet_materials.append((float(k_mu), float(k_lambda), float(k_damp)))
        self.tet_activations.append(0.0)
        return volume

    def add_triangle(self, i, j, k, tri_ke=None, tri_ka=None, tri_kd=None, tri_drag=None, tri_lift=None,
                     **_ignored) -> float:
        """Add a membrane triangle (materials ke, ka, kd, drag, lift); degenerate ones are skipped (returns area)."""
        _, area = triangle_rest_data(np.asarray([self.particle_q[n] for n in (i, j, k)], np.float64),
                                     np.array([[0, 1, 2]]))
        if not area[0] > 0.0:
            return 0.0
        pick = lambda v, d: d if v is None else float(v)
        self.tri_indices.append((int(i), int(j), int(k)))
        self.tri_materials.append((pick(tri_ke, self.default_tri_ke), pick(tri_ka, self.default_tri_ka),
                                   pick(tri_kd, self.default_tri_kd), pick(tri_drag, self.default_tri_drag),
                                   pick(tri_lift, self.default_tri_lift)))
        return float(area[0])

    def add_spring(self, i, j, ke, kd, control=0.0) -> None:
        """Linear spring with rest length from the current positions (Newton ``add_spring``)."""
        rest = float(np.linalg.norm(np.subtract(self.particle_q[i], self.particle_q[j])))
        self.spring_indices.extend((int(i), int(j)))
        self.spring_rest_length.append(rest)
        self.spring_stiffness.append(float(ke))
        self.spring_damping.append(float(kd))

    def add_soft_mesh(self, pos, rot, scale, vel, vertices, indices, density, k_mu, k_lambda, k_damp, **_ignored):
        """Tet4 mesh with lumped density*V/4 masses and one spring per unique edge at (k_mu/2, k_damp/2).

        Restates Newton's ``add_soft_mesh`` (translation/scale; ``rot`` must be the identity
        quaternion here) plus the unique-edge spring network of ``builder.py:51-79``.
        """
        rot = np.asarray(rot, np.float64).reshape(-1)
        if rot.size == 4 and not np.allclose(rot, (0.0, 0.0, 0.0, 1.0)):
            raise NotImplementedError("add_soft_mesh supports the identity rotation only")
        verts = np.asarray(vertices, np.float64).reshape(-1, 3) * float(scale) + np.asarray(pos, np.float64)
        tets = np.asarray(indices, np.int64).reshape(-1, 4)
        start = self.particle_count
        masses = np.zeros(len(verts))
        vols = np.linalg.det((verts[tets[:, 1:]] - verts[tets[:, :1]]).transpose(0, 2, 1)) / 6.0
        for t, vol in zip(tets, vols):
            if vol > 0:
                masses[t] += density * vol / 4.0
        for p, m in zip(verts, masses):
            self.add_particle(p, vel, m)
        first_tet = self.tet_count
        for t in tets:
            self.add_tetrahedron(*(int(n) + start for n in t), k_mu=k_mu, k_lambda=k_lambda, k_damp=k_damp)
        added = set()
        points = np.asarray(self.particle_q)
        for a, b, c, d in self.tet_indices[first_tet:]:
            if np.linalg.det((points[[b, c, d]] - points[a]).T) <= 0.0:
                continue
            for left, right in ((a, b), (a, c), (a, d), (b, c), (b, d), (c, d)):
                key = (min(left, right), max(left, right))
                if key not in added:
                    added.add(key)
                    self.add_spring(key[0], key[1], k_mu * 0.5, k_damp * 0.5, 0.0)

    def add_soft_hex_mesh(self, hex_indices, k_mu=1.0e3, k_lambda=1.0e3, k_damp=0.0) -> None:
        """Q1 Hex8 elements in VTK order (``builder.py:81-93``)."""
        indices = np.asarray(hex_indices, dtype=np.int32)
        if indices.ndim != 2 or indices.shape[1] != 8:
            raise ValueError("hex_indices must have shape (H, 8)")
        if indices.size and (indices.min() < 0 or indices.max() >= self.particle_count):
            raise ValueError("Hex8 indices must reference existing builder particles")
        materials = np.column_stack(
            [np.broadcast_to(np.asarray(v, dtype=np.float32), (len(indices),)) for v in (k_mu, k_lambda, k_damp)]
        )
        if not np.isfinite(materials).all() or np.any(materials < 0):
            raise ValueError("Hex8 materials must be finite and nonnegative")
        self.fem_hex_indices.extend(indices.tolist())
        self.fem_hex_materials.extend(materials.tolist())

    # ---- finalize
    def finalize(self, device="cuda", requires_grad: bool = False) -> Model:
        dev = torch.device(device)
        f32 = dict(dtype=torch.float32, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        m = Model(dev)
        P = self.particle_count
        m.particle_q = torch.tensor(np.asarray(self.particle_q, np.float32).reshape(P, 3), **f32)
        m.particle_qd = torch.tensor(np.asarray(self.particle_qd, np.float32).reshape(P, 3), **f32)
        mass = np.asarray(self.particle_mass, np.float32)
        m.particle_mass = torch.tensor(mass, **f32)
        m.particle_inv_mass = torch.tensor(np.where(mass > 0, 1.0 / np.where(mass > 0, mass, 1), 0).astype(np.float32),
                                           **f32)
        m.particle_radius = torch.tensor(np.asarray(self.particle_radius, np.float32), **f32)
        m.particle_flags = torch.tensor(np.asarray(self.particle_flags, np.int32), **i32)
        m.tet_indices = torch.tensor(np.asarray(self.tet_indices, np.int32).reshape(-1, 4), **i32)
        m.tet_poses = torch.tensor(np.asarray(self.tet_poses, np.float32).reshape(-1, 3, 3), **f32)
        m.tet_materials = torch.tensor(np.asarray(self.tet_materials, np.float32).reshape(-1, 3), **f32)
        m.tet_activations = torch.tensor(np.asarray(self.tet_activations, np.float32), **f32)
        m.spring_indices = torch.tensor(np.asarray(self.spring_indices, np.int32), **i32)
        m.spring_rest_length = torch.tensor(np.asarray(self.spring_rest_length, np.float32), **f32)
        m.spring_stiffness = torch.tensor(np.asarray(self.spring_stiffness, np.float32), **f32)
        m.spring_damping = torch.tensor(np.asarray(self.spring_damping, np.float32), **f32)
        m.gravity = torch.tensor(np.asarray(self.gravity, np.float32), **f32)
        _set_triangles(m, np.asarray(self.particle_q, np.float64).reshape(P, 3), self.tri_indices, self.tri_materials)
        m.particle_grid = HashGrid() if P > 1 else None
        hexes = np.asarray(self.fem_hex_indices, np.int32).reshape(-1, 8)
        inv, det = hex_gauss_data(np.asarray(self.particle_q, np.float64).reshape(P, 3), hexes)
        m.fem = LinearFEMData(
            len(hexes),
            torch.tensor(hexes, **i32),
            torch.tensor(np.asarray(self.fem_hex_materials, np.float32).reshape(-1, 3), **f32),
            torch.tensor(inv.astype(np.float32), **f32),
            torch.tensor(det.astype(np.float32), **f32),
        )
        starts = sorted(set(s for s in self.scene_starts if 0 < s < P))
        m.scene_offsets = np.asarray([0, *starts, P], np.int64) if starts else None
        m.requires_grad = requires_grad
        return m


def _set_triangles(m: Model, x: np.ndarray, tris, materials) -> None:
    tris = np.asarray(tris, np.int32).reshape(-1, 3)
    poses, area = triangle_rest_data(x, tris)
    if np.any(area <= 0.0):
        raise ValueError("triangles must be non-degenerate")
    mats = np.asarray(materials, np.float32).reshape(-1, 5) if len(tris) else np.zeros((0, 5), np.float32)
    if mats.shape != (len(tris), 5):
        raise ValueError("tri_materials must have shape (tri_count, 5): ke, ka, kd, drag, lift")
    dev = m.device
    m.tri_indices = torch.tensor(tris, dtype=torch.int32, device=dev)
    m.tri_poses = torch.tensor(poses.astype(np.float32), dtype=torch.float32, device=dev)
    m.tri_materials = torch.tensor(mats, dtype=torch.float32, device=dev)
    m.tri_areas = torch.tensor(area.astype(np.float32), dtype=torch.float32, device=dev)


def model_from_arrays(
    x,
    mass,
    *,
    tets=None,
    tet_materials=None,
    tris=None,
    tri_materials=None,
    particle_grid=False,
    hexes=None,
    hex_materials=None,
    springs=None,
    spring_ke=None,
    spring_kd=None,
    velocity=None,
    radius=0.0,
    gravity=(0.0, 0.0, -9.81),
    scene_offsets=None,
    device="cuda",
) -> Model:
    """Vectorised builder for large synthetic meshes (same conventions as ``FEMBuilder``)."""
    dev = torch.device(device)
    f32 = dict(dtype=torch.float32, device=dev)
    i32 = dict(dtype=torch.int32, device=dev)
    x = np.asarray(x, np.float64)
    P = len(x)
    m = Model(dev)
    m.particle_q = torch.tensor(x.astype(np.float32), **f32)
    vel = np.zeros((P, 3), np.float32) if velocity is None else np.asarray(velocity, np.float32)
    m.particle_qd = torch.tensor(vel, **f32)
    mass = np.asarray(mass, np.float32)
    m.particle_mass = torch.tensor(mass, **f32)
    m.particle_inv_mass = torch.tensor(np.where(mass > 0, 1.0 / np.where(mass > 0, mass, 1), 0).astype(np.float32),
                                       **f32)
    m.particle_radius = torch.tensor(np.broadcast_to(np.asarray(radius, np.float32), (P,)).copy(), **f32)
    m.particle_flags = torch.ones(P, **i32)
    tets = np.zeros((0, 4), np.int32) if tets is None else np.asarray(tets, np.int32)
    if len(tets):
        Dm = (x[tets[:, 1:]] - x[tets[:, :1]]).transpose(0, 2, 1)
        if np.any(np.linalg.det(Dm) <= 0):
            raise ValueError("tets must be positively oriented")
        poses = np.linalg.inv(Dm).astype(np.float32)
    else:
        poses = np.zeros((0, 3, 3), np.float32)
    m.tet_indices = torch.tensor(tets, **i32)
    m.tet_poses = torch.tensor(poses, **f32)
    mats = np.zeros((0, 3), np.float32) if tet_materials is None or not len(tets) else tet_materials
    m.tet_materials = torch.tensor(np.asarray(mats, np.float32).reshape(-1, 3), **f32)
    m.tet_activations = torch.zeros(len(tets), **f32)
    springs = np.zeros((0, 2), np.int32) if springs is None else np.asarray(springs, np.int32).reshape(-1, 2)
    m.spring_indices = torch.tensor(springs.reshape(-1), **i32)
    rest = np.linalg.norm(x[springs[:, 0]] - x[springs[:, 1]], axis=1) if len(springs) else np.zeros(0)
    m.spring_rest_length = torch.tensor(rest.astype(np.float32), **f32)
    m.spring_stiffness = torch.tensor(np.asarray(spring_ke if spring_ke is not None else [], np.float32), **f32)
    m.spring_damping = torch.tensor(np.asarray(spring_kd if spring_kd is not None else [], np.float32), **f32)
    m.gravity = torch.tensor(np.asarray(gravity, np.float32), **f32)
    hexes = np.zeros((0, 8), np.int32) if hexes is None else np.asarray(hexes, np.int32)
    inv, det = hex_gauss_data(x, hexes)
    m.fem = LinearFEMData(
        len(hexes),
        torch.tensor(hexes, **i32),
        torch.tensor(np.asarray(hex_materials if hex_materials is not None else np.zeros((0, 3)), np.float32)
                     .reshape(-1, 3), **f32),
        torch.tensor(inv.astype(np.float32), **f32),
        torch.tensor(det.astype(np.float32), **f32),
    )
    _set_triangles(m, x, np.zeros((0, 3), np.int32) if tris is None else tris,
                   np.zeros((0, 5)) if tri_materials is None else tri_materials)
    m.particle_grid = HashGrid() if particle_grid else None
    m.scene_offsets = None if scene_offsets is None else np.asarray(scene_offsets, np.int64)
    return m
