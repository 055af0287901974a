"""Seeded synthetic meshes for the SolverFEM hot path (Tet4 / Hex8 grids).

Every workload is generated here with ``numpy.random.default_rng(seed)``; no
dataset is read.  Meshes follow the reference's conventions:

* Hex8 nodes in VTK order (-,-,-), (+,-,-), (+,+,-), (-,+,-), (-,-,+), (+,-,+),
  (+,+,+), (-,+,+) (``_src/geometry/mesh.py:5-7``).
* Tet4 positively oriented, ``det([x1-x0, x2-x0, x3-x0]) > 0``
  (``_src/geometry/mesh.py:8``), from the 6-tet Kuhn/Freudenthal split of each
  cube, which is conforming on a regular grid.
* Lumped masses: Tet4 ``rho*V/4`` per corner, Hex8 ``rho * (weights @ shape)``
  (``tests/fem_fixture.py:22-29``).
* Unique-edge springs in first-seen tet/edge order (``builder.py:51-79``).
* Lame parameters from (E, nu): ``mu = E/(2(1+nu))``,
  ``lambda = E*nu/((1+nu)(1-2nu))``.

The five workloads are the Tet4 cantilever (8x2x2 cubes), the Hex8 64^3 block,
the jittered Tet4 48^3 block with springs, the differentiable 16x4x4 Tet4 beam
and 256 uneven batched scenes.
"""

from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np

HEX_SIGNS = np.array(
    [[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]],
    dtype=np.float64,
)
HEX_CORNERS = ((HEX_SIGNS + 1) // 2).astype(np.int64)


def lame(E: float, nu: float) -> tuple[float, float]:
    """Lame parameters (mu, lambda) of Young's modulus E and Poisson ratio nu."""
    return E / (2.0 * (1.0 + nu)), E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))


def grid_nodes(nx: int, ny: int, nz: int, cell: float, origin=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Node positions of an nx*ny*nz cell grid; node id = i + (nx+1)*(j + (ny+1)*k)."""
    i, j, k = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    pts = np.stack([i, j, k], axis=-1).transpose(2, 1, 0, 3).reshape(-1, 3).astype(np.float64)
    return pts * cell + np.asarray(origin, dtype=np.float64)


def _node_id(nx, ny, i, j, k):
    return i + (nx + 1) * (j + (ny + 1) * k)


def _cell_corners(nx: int, ny: int, nz: int) -> np.ndarray:
    """Node ids of the 8 corners (bit order x, y, z) of every cell, shape [C, 2, 2, 2]."""
    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ci, cj, ck = (a.transpose(2, 1, 0).reshape(-1) for a in (ci, cj, ck))
    out = np.empty((ci.size, 2, 2, 2), dtype=np.int64)
    for bx, by, bz in itertools.product((0, 1), repeat=3):
        out[:, bx, by, bz] = _node_id(nx, ny, ci + bx, cj + by, ck + bz)
    return out


def hex_cells(nx: int, ny: int, nz: int) -> np.ndarray:
    """VTK-ordered Hex8 connectivity of the grid cells, int32 [C, 8]."""
    corners = _cell_corners(nx, ny, nz)
    cols = [corners[:, c[0], c[1], c[2]] for c in HEX_CORNERS]
    return np.stack(cols, axis=1).astype(np.int32)


def kuhn_tets(nx: int, ny: int, nz: int) -> np.ndarray:
    """6-tet Kuhn split of every cell (all share the cell's main diagonal), int32 [6C, 4].

    Each tet walks from corner (0,0,0) to (1,1,1) along one permutation of the
    axes; odd permutations swap the last two vertices to keep det > 0.
    """
    corners = _cell_corners(nx, ny, nz)
    tets = []
    for perm in itertools.permutations(range(3)):
        path = [np.zeros(3, dtype=np.int64)]
        for axis in perm:
            step = path[-1].copy()
            step[axis] = 1
            path.append(step)
        ids = [corners[:, p[0], p[1], p[2]] for p in path]
        sign = np.linalg.det(np.array([path[1] - path[0], path[2] - path[0], path[3] - path[0]], dtype=float).T)
        if sign < 0:
            ids[2], ids[3] = ids[3], ids[2]
        tets.append(np.stack(ids, axis=1))
    # cell-major order: the 6 tets of a cell are consecutive
    return np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)


def tet_volumes(x: np.ndarray, tets: np.ndarray) -> np.ndarray:
    e = x[tets[:, 1:]] - x[tets[:, :1]]
    return np.linalg.det(e.transpose(0, 2, 1)) / 6.0


def tet_poses(x: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """Inverse rest edge matrices ``inv([x1-x0, x2-x0, x3-x0])`` (columns), float32 [T,3,3].

    This is the pose convention that makes ``F = Ds @ pose`` equal I at rest
    (pinned by the reference's ``tests/test_solver.py:213-217``).
    """
    e = (x[tets[:, 1:]] - x[tets[:, :1]]).transpose(0, 2, 1)
    return np.linalg.inv(e).astype(np.float32)


def _hex_shape(points: np.ndarray):
    factors = 1.0 + points[:, None, :] * HEX_SIGNS[None, :, :]
    values = np.prod(factors, axis=2) / 8.0
    deriv = np.empty((len(points), 8, 3))
    for d in range(3):
        other = [a for a in range(3) if a != d]
        deriv[:, :, d] = HEX_SIGNS[None, :, d] * np.prod(factors[:, :, other], axis=2) / 8.0
    return values, deriv


def hex_gauss_points() -> np.ndarray:
    """2x2x2 Gauss points in the builder's order: point g has signs HEX_SIGNS[g] / sqrt(3)."""
    return HEX_SIGNS / np.sqrt(3.0)


def hex_reference_data(x: np.ndarray, hexes: np.ndarray):
    """Per-Gauss-point ``inv_J0`` [H,8,3,3] and ``|det J0|`` [H,8] (float64).

    Follows ``builder.py:95-135``: J0 = sum_a x_a (outer) dN_a/dxi at each point,
    computed in float64 and later stored as float32 (Gauss weight 1 folded in).
    """
    _, deriv = _hex_shape(hex_gauss_points())  # [8 gp, 8 nodes, 3]
    J = np.einsum("hai,gaj->hgij", x[hexes], deriv)
    det = np.linalg.det(J)
    if np.any(det <= 1.0e-12):
        raise ValueError("Degenerate or inverted Hex8 reference Jacobian")
    return np.linalg.inv(J), np.abs(det)


def hex_lumped_mass(x: np.ndarray, hexes: np.ndarray, density: float) -> np.ndarray:
    """Per-node ``density * (weights @ shape)`` summed over elements (``tests/fem_fixture.py:27-29``)."""
    values, _ = _hex_shape(hex_gauss_points())
    _, det = hex_reference_data(x, hexes)
    contrib = density * det @ values  # [H, 8]
    m = np.zeros(len(x))
    np.add.at(m, hexes.ravel(), contrib.ravel())
    return m


def tet_lumped_mass(x: np.ndarray, tets: np.ndarray, density: float) -> np.ndarray:
    m = np.zeros(len(x))
    np.add.at(m, tets.ravel(), np.repeat(density * tet_volumes(x, tets) / 4.0, 4))
    return m


def unique_edges(x: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """Unique tet edges (min, max) in first-seen order, skipping non-positive tets (``builder.py:67-79``)."""
    vol = tet_volumes(x, tets)
    seen = {}
    for t, (a, b, c, d) in enumerate(tets):
        if vol[t] <= 0.0:
            continue
        for left, right in ((a, b), (a, c), (a, d), (b, c), (b, d), (c, d)):
            key = (min(left, right), max(left, right))
            if key not in seen:
                seen[key] = len(seen)
    return np.array(list(seen.keys()), dtype=np.int32).reshape(-1, 2)


@dataclass
class Scene:
    """One synthetic workload, as plain arrays (float64 geometry, float32 material)."""

    name: str
    x: np.ndarray
    mass: np.ndarray
    tets: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))
    tet_materials: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    hexes: np.ndarray = field(default_factory=lambda: np.zeros((0, 8), np.int32))
    hex_materials: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    springs: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))
    spring_ke: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    spring_kd: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    fixed: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    velocity: np.ndarray | None = None
    radius: float = 0.0
    gravity: tuple = (0.0, 0.0, -9.81)
    ground_plane: tuple | None = None
    ground: tuple = (1.0e5, 1.0e2, 1.0e3, 0.5)  # (ke, kd, kf, mu), SolverFEM defaults
    substeps: int = 10
    frames: int = 60
    maxiter: int = 50
    tolerance: float = 1.0e-2
    seed: int = 0
    scene_offsets: np.ndarray | None = None  # node offsets [S+1] for batched scenes
    extra: dict = field(default_factory=dict)

    @property
    def dt(self) -> float:
        return 1.0 / (60.0 * self.substeps)

    @property
    def particle_count(self) -> int:
        return len(self.x)


def tet_block(nx, ny, nz, cell, origin, E, nu, rho, k_damp=0.0):
    x = grid_nodes(nx, ny, nz, cell, origin)
    tets = kuhn_tets(nx, ny, nz)
    mu, lam = lame(E, nu)
    mats = np.tile(np.array([mu, lam, k_damp], np.float32), (len(tets), 1))
    return x, tets, mats, tet_lumped_mass(x, tets, rho)


def hex_block(nx, ny, nz, cell, origin, E, nu, rho, k_damp=0.0):
    x = grid_nodes(nx, ny, nz, cell, origin)
    hexes = hex_cells(nx, ny, nz)
    mu, lam = lame(E, nu)
    mats = np.tile(np.array([mu, lam, k_damp], np.float32), (len(hexes), 1))
    return x, hexes, mats, hex_lumped_mass(x, hexes, rho)


def tet_cantilever(seed: int = 1) -> Scene:
    """8x2x2 cubes of 0.05 m, 6 Tet4 each (192 tets, 81 nodes), x=0 face fixed."""
    x, tets, mats, mass = tet_block(8, 2, 2, 0.05, (0, 0, 0), 1.0e5, 0.45, 1000.0)
    fixed = np.nonzero(np.isclose(x[:, 0], 0.0))[0].astype(np.int32)
    return Scene("tet4_cantilever_8x2x2", x, mass, tets=tets, tet_materials=mats, fixed=fixed,
                 substeps=10, frames=60, maxiter=50, seed=seed)


# The ground is an explicit penalty force (kernels.py:1132-1195).  With 1 cm
# cells the node masses are 0.14-1.1 g, and at h = 1/600 s the solver's default
# penalty (ke 1e5 N/m, kd 1e2 N s/m) and even ke 1e3 / kd 1 diverge within a few
# frames, in this restatement of the algorithm as in the reference's.  The
# ground-contact workloads therefore use the stiffest penalty found stable over
# 30 frames: ke 300 N/m, no normal damping, kf 1e3, Coulomb mu 0.5.
STABLE_GROUND_1CM = (300.0, 0.0, 1.0e3, 0.5)


def hex_block_64(n: int = 64, seed: int = 2) -> Scene:
    """n^3 Hex8 cells of 1 cm resting on the ground, velocities N(0, 0.05) per component."""
    x, hexes, mats, mass = hex_block(n, n, n, 0.01, (0, 0, 0), 5.0e5, 0.4, 1100.0)
    rng = np.random.default_rng(seed)
    vel = rng.normal(0.0, 0.05, size=x.shape).astype(np.float32)
    return Scene(f"hex8_block_{n}^3", x, mass, hexes=hexes, hex_materials=mats, velocity=vel,
                 ground_plane=(0.0, 0.0, 1.0, 0.0), ground=STABLE_GROUND_1CM, substeps=10, frames=30, maxiter=50,
                 seed=seed)


def tet_jittered_48(n: int = 48, seed: int = 3) -> Scene:
    """n^3 jittered Tet4 block (1 cm cells, +/-0.2 cell interior jitter) with edge springs, dropped from 0.2 m."""
    cell = 0.01
    x = grid_nodes(n, n, n, cell, (0.0, 0.0, 0.2))
    rng = np.random.default_rng(seed)
    ijk = np.rint((x - (0.0, 0.0, 0.2)) / cell).astype(np.int64)
    interior = np.all((ijk > 0) & (ijk < n), axis=1)
    jitter = rng.uniform(-0.2 * cell, 0.2 * cell, size=x.shape)
    x[interior] += jitter[interior]
    tets = kuhn_tets(n, n, n)
    mu, lam = lame(2.0e5, 0.45)
    mats = np.tile(np.array([mu, lam, 0.0], np.float32), (len(tets), 1))
    mass = tet_lumped_mass(x, tets, 1000.0)
    springs = unique_edges(x, tets)
    ke = np.full(len(springs), 1.0e3, np.float32)
    kd = np.full(len(springs), 0.1, np.float32)
    return Scene(f"tet4_jittered_{n}^3", x, mass, tets=tets, tet_materials=mats, springs=springs,
                 spring_ke=ke, spring_kd=kd, ground_plane=(0.0, 0.0, 1.0, 0.0), ground=STABLE_GROUND_1CM,
                 substeps=10, frames=60, maxiter=50, seed=seed)


def tet_beam(seed: int = 4) -> Scene:
    """16x4x4 cubes of 0.05 m x 6 tets (1,536 tets, 425 nodes) hanging from its fixed top end, mu scale U[0.8,1.2].

    The beam's long axis is z: the 25 nodes of the top face (z = 0.8 m) are
    fixed and the tip face is z = 0, with gravity along the axis.  The
    differentiable contract assembles A once at the rest pose, so the workload
    must stay in small strain with 30 CG iterations converging from zero.  A
    cantilever under gravity cannot do both at h = 1/240 (its tip sag times
    h^2 E / (rho cell^2) is about 1 m whatever E is); the hanging beam stretches
    by about rho g L^2 / 2E = 3 cm, oscillates 1-6 cm below rest, and CG
    reaches a relative residual of 1e-6 in 30 iterations.  The target is 0.05 m
    below the tip face's rest centroid.
    """
    x, tets, mats, mass = tet_block(4, 4, 16, 0.05, (0, 0, 0), 1.0e5, 0.45, 1000.0)
    rng = np.random.default_rng(seed)
    scale = rng.uniform(0.8, 1.2, size=len(tets)).astype(np.float32)
    fixed = np.nonzero(np.isclose(x[:, 2], x[:, 2].max()))[0].astype(np.int32)
    tip = np.nonzero(np.isclose(x[:, 2], 0.0))[0].astype(np.int32)
    target = x[tip].mean(axis=0) - np.array([0.0, 0.0, 0.05])
    return Scene("tet4_beam_16x4x4", x, mass, tets=tets, tet_materials=mats, fixed=fixed, substeps=4,
                 frames=120, maxiter=30, seed=seed,
                 extra={"mu_scale": scale, "tip_nodes": tip, "target": target, "checkpoint_every": 10})


def batched_scenes(count: int = 256, seed: int = 5, cell: float = 0.05, dims=(4, 32)) -> Scene:
    """``count`` independent meshes (half Tet4, half Hex8) with per-axis dims U{lo..hi}, one x=0 face fixed each.

    Every mesh is built at the origin: the scenes do not interact, and the Hex8
    deformation gradient sums absolute node positions times shape gradients
    (kernels.py:1551-1560), so in float32 its error grows with the distance from
    the origin over the cell size (a mesh 235 m out with 5 cm cells loses about
    four digits of F).
    """
    rng = np.random.default_rng(seed)
    xs, masses, tets, tmats, hexes, hmats, fixed, offsets = [], [], [], [], [], [], [], [0]
    for s in range(count):
        nx, ny, nz = (int(v) for v in rng.integers(dims[0], dims[1] + 1, size=3))
        E = float(np.exp(rng.uniform(np.log(1.0e4), np.log(1.0e6))))
        nu = float(rng.uniform(0.3, 0.48))
        origin = (0.0, 0.0, 0.0)
        base = offsets[-1]
        if s % 2 == 0:
            x, el, mats, mass = tet_block(nx, ny, nz, cell, origin, E, nu, 1000.0)
            tets.append(el + base)
            tmats.append(mats)
        else:
            x, el, mats, mass = hex_block(nx, ny, nz, cell, origin, E, nu, 1000.0)
            hexes.append(el + base)
            hmats.append(mats)
        fixed.append(np.nonzero(np.isclose(x[:, 0], 0.0))[0].astype(np.int32) + base)
        xs.append(x)
        masses.append(mass)
        offsets.append(base + len(x))
    cat = lambda parts, shape, dtype: np.concatenate(parts).astype(dtype) if parts else np.zeros(shape, dtype)  # noqa: E731
    return Scene(
        f"batched_{count}_scenes",
        np.concatenate(xs),
        np.concatenate(masses),
        tets=cat(tets, (0, 4), np.int32),
        tet_materials=cat(tmats, (0, 3), np.float32),
        hexes=cat(hexes, (0, 8), np.int32),
        hex_materials=cat(hmats, (0, 3), np.float32),
        fixed=np.concatenate(fixed).astype(np.int32),
        substeps=10,
        frames=60,
        maxiter=50,
        seed=seed,
        scene_offsets=np.asarray(offsets, dtype=np.int64),
    )


def split_batched(scene: Scene) -> list[Scene]:
    """The independent scenes of a batched Scene, each re-indexed from node 0."""
    out = []
    offs = scene.scene_offsets
    for s in range(len(offs) - 1):
        lo, hi = int(offs[s]), int(offs[s + 1])
        tsel = np.all((scene.tets >= lo) & (scene.tets < hi), axis=1) if len(scene.tets) else np.zeros(0, bool)
        hsel = np.all((scene.hexes >= lo) & (scene.hexes < hi), axis=1) if len(scene.hexes) else np.zeros(0, bool)
        fixed = scene.fixed[(scene.fixed >= lo) & (scene.fixed < hi)] - lo
        out.append(Scene(
            f"{scene.name}[{s}]", scene.x[lo:hi], scene.mass[lo:hi],
            tets=(scene.tets[tsel] - lo).astype(np.int32) if tsel.any() else np.zeros((0, 4), np.int32),
            tet_materials=scene.tet_materials[tsel] if tsel.any() else np.zeros((0, 3), np.float32),
            hexes=(scene.hexes[hsel] - lo).astype(np.int32) if hsel.any() else np.zeros((0, 8), np.int32),
            hex_materials=scene.hex_materials[hsel] if hsel.any() else np.zeros((0, 3), np.float32),
            fixed=fixed.astype(np.int32), gravity=scene.gravity, substeps=scene.substeps, frames=scene.frames,
            maxiter=scene.maxiter, tolerance=scene.tolerance, seed=scene.seed))
    return out


CONFIGS = {
    "tet4_cantilever": tet_cantilever,
    "hex8_block": hex_block_64,
    "tet4_jittered": tet_jittered_48,
    "tet4_beam": tet_beam,
    "batched": batched_scenes,
}
