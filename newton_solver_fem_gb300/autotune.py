"""Autotuner for the persistent PCG kernel's launch variant and the standalone SpMV.

PCG axes (``fem_set_tuning`` keys):

* staging depth -- ``FEM_TUNE_SPMV_UNROLL``: block columns whose loads are in
  flight per thread before any is used (1, 2, 4);
* rows per CTA -- ``FEM_TUNE_CTA_THREADS``: 256, 512 or 1024 threads per
  persistent CTA; the grid is as many CTAs as stay co-resident, so this sets
  how many 32-row slices each CTA owns (its share of the rows and of the grid
  reductions);
* the CG recurrence -- ``FEM_TUNE_CG_VARIANT``: standard (two grid reductions
  per iteration) or single-reduction Chronopoulos-Gear;
* the matrix bytes held in L2 (``FEM_TUNE_L2_RESIDENT_BYTES``): the automatic
  rule (-2: the whole matrix when it fits in 60% of L2, else none) won every
  measurement, so candidates keep it.

Warps per row: the matrix is SELL-32 with one lane per row (a warp streams the
same column slot of 32 rows, coalesced), so each row has exactly one thread;
the staging depth is the knob that sets how much of a row is in flight.

For a solver and a frame function the tuner restores the same initial state
for every candidate, runs one warm-up frame, then times the PCG launches of
``frames`` eager frames with per-launch CUDA events.  It scores each candidate
by microseconds per CG iteration, so that candidates with different iteration
counts compare fairly, and applies the best one.  Results are cached in a JSON
file keyed by GPU name and problem signature (nodes, stored blocks, scenes).

The standalone SpMV (``fem_apply_operator``) has its own axes:
``FEM_TUNE_OPERATOR_BATCH`` (block columns in flight per thread: 2 at 32
registers or 4 at 48) and ``FEM_TUNE_OPERATOR_STAGE`` (0: direct loads; 4 or 8:
the block planes staged through shared memory by bulk asynchronous copies of
that many block columns); ``tune_operator`` times each candidate after an L2
flush.

Command line (prints one JSON record per candidate, then the choice)::

    python -m newton_solver_fem_gb300.autotune --cells 64
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
from pathlib import Path

import torch

from . import _lib

AXES = {
    "unroll": _lib.FEM_TUNE_SPMV_UNROLL,
    "threads": _lib.FEM_TUNE_CTA_THREADS,
    "cg_variant": _lib.FEM_TUNE_CG_VARIANT,
    "resident_bytes": _lib.FEM_TUNE_L2_RESIDENT_BYTES,
}
# every staging depth at every CTA size with the standard recurrence, plus the single-reduction
# recurrence at the default shape
DEFAULT_CANDIDATES = [dict(unroll=u, threads=t, cg_variant=0, resident_bytes=-2)
                      for t in (1024, 512, 256) for u in (4, 2, 1)] + \
                     [dict(unroll=u, threads=1024, cg_variant=1, resident_bytes=-2) for u in (4, 2)]
CACHE = Path(os.environ.get("FEM_GB300_TUNE_CACHE", Path.home() / ".cache" / "fem_gb300_tune.json"))


def _key(solver) -> str:
    info = solver.matrix_info()
    name = torch.cuda.get_device_name(solver.device)
    return f"{name}|P={solver.model.particle_count}|blocks={info['stored_blocks']}|S={solver.model.scene_count}"


def apply(solver, choice: dict) -> None:
    """Set every tuning key named in ``choice`` (axis name -> value)."""
    lib = _lib.load()
    for name, value in choice.items():
        if name in AXES:
            _lib.check(lib.fem_set_tuning(solver._handle, AXES[name], int(value)))


def current(solver) -> dict:
    lib = _lib.load()
    out = {}
    for name, key in (*AXES.items(), ("resident_slices", _lib.FEM_TUNE_RESIDENT_SLICES), ("grid", _lib.FEM_TUNE_GRID)):
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
    """Pick and apply the fastest PCG launch variant for this solver; returns the chosen record with the
    measured records of every candidate under ``"candidates"``."""
    key = _key(solver)
    cache = {}
    if use_cache and CACHE.exists():
        try:
            cache = json.loads(CACHE.read_text())
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        best = cache[key]
        apply(solver, {k: v for k, v in best.items() if k in AXES})
        return best
    records = []
    for cand in candidates or DEFAULT_CANDIDATES:
        apply(solver, cand)
        rec = {**current(solver), **measure(solver, frame, restore, frames)}
        records.append(rec)
        if verbose:
            print(json.dumps(rec), flush=True)
    best = dict(min(records, key=lambda r: r["us_per_iteration"]))
    apply(solver, {k: v for k, v in best.items() if k in AXES})
    best["candidates"] = records
    if use_cache:
        cache[key] = best
        try:
            CACHE.parent.mkdir(parents=True, exist_ok=True)
            CACHE.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return best


def time_operator(solver, repeats: int = 21) -> float:
    """Median microseconds of one fem_apply_operator after an L2 flush (write, then a clean read)."""
    lib = _lib.load()
    P = solver.model.particle_count
    g = torch.Generator(device=solver.device).manual_seed(0)
    x = torch.randn((P, 3), device=solver.device, generator=g)
    y = torch.empty_like(x)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=solver.device)
    clean = torch.ones(128 << 20, dtype=torch.float32, device=solver.device)
    stream = torch.cuda.current_stream(solver.device)
    times = []
    for _ in range(repeats):
        flush.fill_(1)
        clean.sum()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _lib.check(lib.fem_apply_operator(solver._handle, x.data_ptr(), y.data_ptr(), stream.cuda_stream))
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    return 1e3 * statistics.median(times[1:])


OPERATOR_AXES = {"operator_batch": _lib.FEM_TUNE_OPERATOR_BATCH, "operator_stage": _lib.FEM_TUNE_OPERATOR_STAGE}
# direct loads with 2 or 4 block columns in flight, and the planes staged through shared memory by bulk
# copies of 4 or 8 block columns
OPERATOR_CANDIDATES = [dict(operator_batch=2, operator_stage=0), dict(operator_batch=4, operator_stage=0),
                       dict(operator_batch=2, operator_stage=4), dict(operator_batch=2, operator_stage=8)]


def tune_operator(solver, candidates=None, timer=None) -> dict:
    """Pick and apply the fastest fem_apply_operator variant (FEM_TUNE_OPERATOR_BATCH and
    FEM_TUNE_OPERATOR_STAGE); returns the chosen keys with "us", and every candidate's record."""
    lib = _lib.load()
    timer = timer or time_operator

    def set_keys(choice):
        for name, key in OPERATOR_AXES.items():
            _lib.check(lib.fem_set_tuning(solver._handle, key, int(choice[name])))

    records = []
    for cand in candidates or OPERATOR_CANDIDATES:
        set_keys(cand)
        records.append({**{k: int(v) for k, v in cand.items()}, "us": timer(solver)})
    best = min(records, key=lambda r: r["us"])
    set_keys(best)
    return {**best, "candidates": records}


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
    op = tune_operator(solver)
    print(json.dumps({"best": {k: v for k, v in best.items() if k != "candidates"}, "operator": op}))


if __name__ == "__main__":
    main()
