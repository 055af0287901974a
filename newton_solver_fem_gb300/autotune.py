"""Autotuner for the persistent PCG kernel's launch variant.

Tunables (``fem_set_tuning``): the SpMV unroll (block columns in flight per
thread: 1, 2, 4), the threads per persistent CTA (256, 512, 1024: the grid is
as many CTAs as stay co-resident) and the matrix bytes loaded with the L2
evict_last policy.  Pinning part of a matrix larger than L2 lost every time,
and pinning a whole matrix that fits won, so the default candidates use the
automatic rule (-2: the whole matrix when it fits in 60% of L2, else none).
For a solver and a frame function the tuner restores the same initial state
for every candidate, runs one warm-up frame, then times the PCG launches of
``frames`` eager frames with per-launch CUDA events.  It scores each candidate
by microseconds per CG iteration, so that candidates with different iteration
counts compare fairly, and applies the best one.  Results are cached in a JSON
file keyed by GPU name and problem signature (nodes, stored blocks, scenes).

Command line (prints one JSON record per candidate, then the choice)::

    python -m newton_solver_fem_gb300.autotune --cells 64
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
from pathlib import Path

import torch

from . import _lib

# (unroll, CTA threads, L2-resident bytes)
DEFAULT_CANDIDATES = [(u, t, -2) for t in (1024, 512, 256) for u in (4, 2)] + [(1, 1024, -2)]
CACHE = Path(os.environ.get("FEM_GB300_TUNE_CACHE", Path.home() / ".cache" / "fem_gb300_tune.json"))


def _key(solver) -> str:
    info = solver.matrix_info()
    name = torch.cuda.get_device_name(solver.device)
    return f"{name}|P={solver.model.particle_count}|blocks={info['stored_blocks']}|S={solver.model.scene_count}"


def apply(solver, unroll: int, threads: int, resident_bytes: int) -> None:
    lib = _lib.load()
    _lib.check(lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_SPMV_UNROLL, int(unroll)))
    _lib.check(lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_CTA_THREADS, int(threads)))
    _lib.check(lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_L2_RESIDENT_BYTES, int(resident_bytes)))


def current(solver) -> dict:
    lib = _lib.load()
    out = {}
    for name, key in (("unroll", _lib.FEM_TUNE_SPMV_UNROLL), ("threads", _lib.FEM_TUNE_CTA_THREADS),
                      ("resident_bytes", _lib.FEM_TUNE_L2_RESIDENT_BYTES),
                      ("resident_slices", _lib.FEM_TUNE_RESIDENT_SLICES), ("grid", _lib.FEM_TUNE_GRID)):
        v = ctypes.c_int64()
        _lib.check(lib.fem_get_tuning(solver._handle, key, ctypes.byref(v)))
        out[name] = v.value
    return out


def measure(solver, frame, restore, frames: int = 3) -> dict:
    """Time the PCG launches of ``frames`` eager frames after one warm-up frame."""
    lib = _lib.load()
    restore()
    frame()
    torch.cuda.synchronize()
    s0 = solver.stats()
    _lib.check(lib.fem_set_timing(solver._handle, 1))
    for _ in range(frames):
        frame()
    t_ms, n = ctypes.c_double(), ctypes.c_int64()
    _lib.check(lib.fem_get_timing(solver._handle, ctypes.byref(t_ms), ctypes.byref(n)))
    _lib.check(lib.fem_set_timing(solver._handle, 0))
    s1 = solver.stats()
    launches = max(1, n.value)
    iters = (s1["total_iterations"] - s0["total_iterations"]) / launches
    launch_ms = t_ms.value / launches
    return {"launch_ms": launch_ms, "iterations": iters, "us_per_iteration": 1e3 * launch_ms / (iters + 1.0)}


def autotune(solver, frame, restore, candidates=None, frames: int = 3, use_cache: bool = True,
             verbose: bool = False) -> dict:
    """Pick and apply the fastest (unroll, CTA threads, resident bytes) for this solver; returns the record."""
    key = _key(solver)
    cache = {}
    if use_cache and CACHE.exists():
        try:
            cache = json.loads(CACHE.read_text())
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        best = cache[key]
        apply(solver, best["unroll"], best.get("threads", 1024), best["resident_bytes"])
        return best
    records = []
    for unroll, threads, resident in candidates or DEFAULT_CANDIDATES:
        apply(solver, unroll, threads, resident)
        rec = {**current(solver), **measure(solver, frame, restore, frames)}
        records.append(rec)
        if verbose:
            print(json.dumps(rec), flush=True)
    best = min(records, key=lambda r: r["us_per_iteration"])
    apply(solver, best["unroll"], best["threads"], best["resident_bytes"])
    if use_cache:
        cache[key] = best
        try:
            CACHE.parent.mkdir(parents=True, exist_ok=True)
            CACHE.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return best


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--cells", type=int, default=64)
    p.add_argument("--frames", type=int, default=3)
    args = p.parse_args()
    from . import SolverFEM, model_from_arrays, scenes

    sc = scenes.hex_block_64(n=args.cells)
    model = model_from_arrays(sc.x, sc.mass, hexes=sc.hexes, hex_materials=sc.hex_materials, velocity=sc.velocity,
                              radius=0.0, gravity=sc.gravity, device="cuda:0")
    ke, kd, kf, mu = sc.ground
    solver = SolverFEM(model, dt=sc.dt, solver_type="cg", preconditioner_type="block_diag",
                       linear_solver_maxiter=sc.maxiter, linear_solver_tolerance=sc.tolerance,
                       ground_plane=sc.ground_plane, ground_ke=ke, ground_kd=kd, ground_kf=kf, ground_mu=mu,
                       self_contact_ke=0.0)
    s0, s1 = model.state(), model.state()
    q0, v0 = model.particle_q.clone(), model.particle_qd.clone()

    def restore():
        s0.particle_q.copy_(q0)
        s0.particle_qd.copy_(v0)
        solver.reset()

    def frame():
        a, b = s0, s1
        solver.refresh_tangent(a.particle_q)
        for _ in range(sc.substeps):
            solver.step(a, b, None, None, sc.dt)
            a, b = b, a

    best = autotune(solver, frame, restore, frames=args.frames, use_cache=False, verbose=True)
    print(json.dumps({"best": best}))


if __name__ == "__main__":
    main()
