"""Regenerate ``beam_fd.npz``: float64 central differences of the differentiable-beam loss.

Workload: 16x4x4 cubes of 0.05 m x 6 Tet4 (1,536 tets, 425 nodes) hanging
from its fixed top face, per-element shear scale U[0.8, 1.2] (seeded), gravity,
120 frames x 4 substeps (h = 1/240 s).  Loss = squared distance from the tip-face centroid
to a target 0.05 m below its rest position.  The matrix is assembled once at
the rest pose with the nominal scales and held fixed (the differentiable
contract: no dA/dtheta), and every solve runs from zero to a relative residual
of 1e-13, so the differences are those of the converged linear solve.

Sixteen seeded parameters: 8 per-element scales and 8 initial-velocity
components of free nodes, each differenced with eps = 1e-3 (and 5e-4 as a
truncation check: the two must agree to 1e-4 relative).  Runs the float64
oracle only; takes a few minutes on 8 cores::

    python tests/golden/make_beam_fd.py
"""

import multiprocessing as mp
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from newton_solver_fem_gb300 import scenes  # noqa: E402
from oracle import fem_oracle as O  # noqa: E402

OUT = Path(__file__).with_name("beam_fd.npz")
EPS = (1.0e-3, 5.0e-4)
PARAM_SEED = 404


def beam_inputs():
    """The beam as float32-rounded float64 arrays (what the GPU solver sees)."""
    sc = scenes.tet_beam()
    r = lambda a: np.asarray(a, np.float32).astype(np.float64)  # noqa: E731
    poses = scenes.tet_poses(sc.x, sc.tets).astype(np.float32)
    return sc, r(sc.x), r(sc.mass), poses, r(sc.extra["mu_scale"])


def parameters(sc):
    """(kind, index, axis) for 8 element scales and 8 initial-velocity components of free nodes."""
    rng = np.random.default_rng(PARAM_SEED)
    elems = np.sort(rng.choice(len(sc.tets), size=8, replace=False))
    free = np.setdiff1d(np.arange(len(sc.x)), sc.fixed)
    nodes = np.sort(rng.choice(free, size=8, replace=False))
    axes = rng.integers(0, 3, size=8)
    kind = np.array([0] * 8 + [1] * 8, np.int32)  # 0: mu scale, 1: initial velocity
    index = np.concatenate([elems, nodes]).astype(np.int32)
    axis = np.concatenate([np.zeros(8, np.int64), axes]).astype(np.int32)
    return kind, index, axis


def rollout(scale, v0):
    sc, x, m, poses, scale0 = beam_inputs()
    o = O.OracleFEM(x, m, tets=sc.tets, tet_poses=poses, tet_materials=sc.tet_materials.astype(np.float32),
                    fixed=sc.fixed, dt=sc.dt, maxiter=400, tolerance=1.0e-13, mu_scale=scale0)
    o.mu_scale = scale  # forces see the perturbed scale; the matrix stays at the nominal one
    q, v = x.copy(), v0.copy()
    for _ in range(sc.frames * sc.substeps):
        o.dv[:] = 0.0
        q, v, _ = o.step(q, v, sc.dt)
    centroid = q[sc.extra["tip_nodes"]].mean(axis=0)
    return float(np.sum((centroid - sc.extra["target"]) ** 2))


def _job(args):
    kind, index, axis, delta = args
    sc, x, _, _, scale0 = beam_inputs()
    scale = scale0.copy()
    v0 = np.zeros_like(x)
    if kind == 0:
        scale[index] += delta
    elif kind == 1:
        v0[index, axis] += delta
    return rollout(scale, v0)


def main():
    sc, x, _, _, scale0 = beam_inputs()
    kind, index, axis = parameters(sc)
    jobs = [(0, 0, 0, 0.0)]
    for eps in EPS:
        for k, i, a in zip(kind, index, axis):
            jobs += [(int(k), int(i), int(a), eps), (int(k), int(i), int(a), -eps)]
    with mp.get_context("spawn").Pool() as pool:
        values = pool.map(_job, jobs)
    loss = values[0]
    fd = []
    for e, eps in enumerate(EPS):
        vals = np.asarray(values[1 + 32 * e: 1 + 32 * (e + 1)]).reshape(16, 2)
        fd.append((vals[:, 0] - vals[:, 1]) / (2.0 * eps))
    fd = np.asarray(fd)
    spread = np.abs(fd[0] - fd[1]) / np.maximum(np.abs(fd[0]), 1e-12)
    if np.max(spread) > 1.0e-4:
        raise SystemExit(f"finite differences not converged in eps: {spread}")
    np.savez(OUT, loss=loss, fd=fd[0], fd_half_eps=fd[1], kind=kind, index=index, axis=axis,
             mu_scale=scale0.astype(np.float32), eps=np.asarray(EPS))
    print(f"loss {loss:.9e}")
    for k, i, a, g in zip(kind, index, axis, fd[0]):
        print(("scale" if k == 0 else "v0"), i, a, f"{g:.9e}")


if __name__ == "__main__":
    main()
