#!/usr/bin/env python
"""Benchmark of the SolverFEM hot path on GB300: DOF-substeps/s of the Hex8 64^3 block.

Workload (the single-GPU configuration the metric is quoted on): a 64^3 Q1
Hex8 grid of 1 cm cells (262,144 elements, 274,625 nodes, 823,875 DOF),
E = 5e5 Pa, nu = 0.4, rho = 1100, resting on the analytic ground (mu = 0.5),
velocities seeded N(0, 0.05 m/s); 60 Hz frames of 10 substeps; CG with
block-Jacobi at relative residual 1e-2, at most 50 iterations; float32.

One bench step = one frame = tangent refresh + 10 linearly implicit substeps,
replayed from a captured CUDA graph.  ``value`` = 3 * nodes * substeps / frame
time with inputs resident in HBM.  ``e2e`` = the same metric through the
public ``SolverFEM`` API with the frame's positions/velocities copied from
pinned host memory and the result read back every frame; each frame is an
eager ``refresh_tangent`` and a captured graph of the substeps' ``step`` calls,
the way the reference's example drives its solver.  ``roofline`` = the
persistent PCG kernel's algorithmic bytes per launch over its CUDA-event launch
time.  ``cpu_baseline`` = the float32 C/OpenMP port of the reference algorithm
(``oracle/fem_port.c``, checked against the float64 NumPy oracle by the tests)
on all host cores, on a bounded sample of the same workload.

``--impl reference`` times that C/OpenMP port alone on the same metric and
config (the reference itself needs Warp and Newton, which cannot be installed
in this image).  Multi-GPU: the single mesh does not shard, so N GPUs run N
independent replicas ("replicas only"); value = all replicas' DOF-substeps / max
time over ranks.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "DOF-substeps/s at rel-res 1e-2: batched/adjoint vs plain on 1 GB300; SpMV GB/s"
UNIT = "DOF-substeps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    p.add_argument("--cells", type=int, default=64, help="Hex8 cells per axis (64 = the benchmark workload)")
    p.add_argument("--cpu-sample", type=float, default=20.0, help="seconds budget for the CPU baseline sample")
    p.add_argument("--cpu-cells", type=int, default=None, help="Hex8 cells per axis of the CPU sample (default: same)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-batched", action="store_true", help="skip the 256-scene batched vs plain measurement")
    p.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-beam gradient measurement")
    p.add_argument("--no-tet", action="store_true", help="skip the jittered Tet4 48^3 measurement")
    p.add_argument("--profile-workload", choices=("batched", "tet", "hex"), default=None,
                   help="run only --steps eager frames of the 256-scene batch, the jittered Tet4 48^3 block or the "
                        "Hex8 block (--cells), print their time and the CG iterations of every PCG launch, and exit "
                        "(a target for ncu captures; no JSON line)")
    p.add_argument("--trace-iterations", action="store_true",
                   help="print the CG iterations of every PCG launch of the eager warm-up frame to stderr "
                        "(maps an ncu launch index to its iteration count)")
    return p.parse_args()


def peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        d = json.loads(path.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dram_traffic_per_launch(iterations: float):
    """Measured DRAM bytes (read + write) of one PCG launch at this mean iteration count.

    From the committed ncu summary of two full 64^3 launches (18 and 22 CG iterations):
    ``dram_bytes_fit: <prologue+epilogue bytes> <bytes per iteration>``.  None when absent.
    """
    path = ROOT / "profiles" / "pcg_kernel_hex8_64_dram.md"
    if not path.exists():
        return None
    for line in path.read_text().splitlines():
        if line.strip().startswith("dram_bytes_fit:"):
            try:
                base, per_iter = (float(v) for v in line.split(":", 1)[1].split()[:2])
            except ValueError:
                return None
            return base + per_iter * iterations
    return None


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [c.strip() for c in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for name, val in zip(names, r[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(cells: int, device: str):
    import numpy as np

    from newton_solver_fem_gb300 import SolverFEM, model_from_arrays, scenes

    sc = scenes.hex_block_64(n=cells)
    model = model_from_arrays(sc.x, sc.mass, hexes=sc.hexes, hex_materials=sc.hex_materials, velocity=sc.velocity,
                              radius=0.0, gravity=sc.gravity, device=device)
    ke, kd, kf, mu = sc.ground
    solver = SolverFEM(model, dt=sc.dt, solver_type="cg", preconditioner_type="block_diag",
                       linear_solver_maxiter=sc.maxiter, linear_solver_tolerance=sc.tolerance,
                       ground_plane=sc.ground_plane, ground_ke=ke, ground_kd=kd, ground_kf=kf, ground_mu=mu,
                       self_contact_ke=0.0)
    return sc, model, solver, np


def spmv_bytes(nnzb: int, n: int, col_bytes: float = 4) -> float:
    """Algorithmic bytes of one 3x3-BSR SpMV: 36 B values + the column index per block (4 B, 2 B as a
    16-bit offset from the row, or on average less where a slice's rows share one offset), offsets,
    x read, y write."""
    return (36 + col_bytes) * nnzb + 4 * (n + 1) + 24 * n


def pcg_launch_bytes(nnzb: int, n: int, iterations: float, col_bytes: float = 4) -> float:
    """Algorithmic bytes of one persistent PCG launch.

    Per CG iteration: one SpMV plus 120 B/node (Minv 36, read x r p Ap 48, write x r p 36).
    Prologue (predictor and initial residual in one pass over A): one SpMV plus
    read v, dv, f and write f, r (60 B/node) plus read x, r, f, Minv and write x, r, z (108 B/node).
    Epilogue: read x, v, q and write dv, q, v (72 B/node).
    """
    sp = spmv_bytes(nnzb, n, col_bytes)
    return iterations * (sp + 120 * n) + sp + (60 + 108 + 72) * n


def cpu_port(cells: int):
    """The C/OpenMP port of the reference algorithm on the same workload (setup is untimed)."""
    import numpy as np

    from newton_solver_fem_gb300 import scenes
    from oracle import fem_oracle as O
    from oracle import fem_port

    sc = scenes.hex_block_64(n=cells)
    x = sc.x.astype(np.float32).astype(np.float64)
    inv, det = O.hex_builder_data(x, sc.hexes)
    port = fem_port.PortFEM(x, sc.mass.astype(np.float32), hexes=sc.hexes, hex_inv_J0=inv.astype(np.float32),
                            hex_det_J0_w=det.astype(np.float32), hex_materials=sc.hex_materials, dt=sc.dt,
                            ground_plane=sc.ground_plane, ground=sc.ground, maxiter=sc.maxiter,
                            tolerance=sc.tolerance)
    return sc, port, x.astype(np.float32), sc.velocity.astype(np.float32), fem_port.threads()


def port_frame(sc, port, q, v, max_substeps=None, budget_s=None):
    """One frame (tangent refresh + substeps); returns (q, v, seconds, substeps run)."""
    t0 = time.perf_counter()
    q = port.refresh_tangent(q)
    subs = 0
    while subs < sc.substeps:
        if max_substeps is not None and subs >= max_substeps:
            break
        if budget_s is not None and subs > 0 and time.perf_counter() - t0 > budget_s:
            break
        q, v, _ = port.step(q, v, sc.dt)
        subs += 1
    return q, v, time.perf_counter() - t0, subs


def cpu_baseline(cells: int, budget_s: float) -> dict:
    """C/OpenMP port on the host cores: one frame of the same workload, cut at the time budget."""
    sc, port, q, v, cores = cpu_port(cells)
    t_sub0 = time.perf_counter()
    q = port.refresh_tangent(q)
    t_refresh = time.perf_counter() - t_sub0
    subs, t_sub = 0, 0.0
    while subs < sc.substeps and (subs == 0 or t_refresh + t_sub < budget_s):
        t1 = time.perf_counter()
        q, v, _ = port.step(q, v, sc.dt)
        t_sub += time.perf_counter() - t1
        subs += 1
    frame_s = t_refresh + t_sub / subs * sc.substeps
    value = 3 * port.n * sc.substeps / frame_s
    return {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"C/OpenMP port ({cores} threads), Hex8 {cells}^3: 1 tangent refresh + {subs} substep(s) "
                      f"({t_refresh + t_sub:.1f} s); frame = refresh + 10 x mean substep"}


def run_reference(args) -> None:
    """CPU arm: the C/OpenMP restatement of the reference path, one frame per step on all host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sc, port, q, v, cores = cpu_port(args.cells)
    for _ in range(args.warmup):  # each warm-up step is one substep, to page in and settle the caches
        q, v, _ = port.step(q, v, sc.dt)
    times = []
    for _ in range(args.steps):
        q, v, sec, subs = port_frame(sc, port, q, v)
        times.append(sec)
    frame_s = statistics.median(times)
    value = 3 * port.n * sc.substeps / frame_s
    base = {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"C/OpenMP port ({cores} threads): {args.steps} full frames (refresh + 10 substeps) of "
                      f"Hex8 {args.cells}^3, median"}
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": frame_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"hex8_block_{args.cells}^3", "nodes": port.n, "substeps_per_step": sc.substeps,
                   "cg_tol": sc.tolerance, "cg_maxiter": sc.maxiter, "preconditioner": "block_diag"},
        "cpu_baseline": base,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference needs Warp 1.17 + Newton 1.7 (not installable in this image); this arm times the "
                "CPU restatement of its algorithm",
    }
    print(json.dumps(line), flush=True)


def scene_solver(sc, device, scene_offsets=None):
    from newton_solver_fem_gb300 import SolverFEM, model_from_arrays

    model = model_from_arrays(sc.x, sc.mass, tets=sc.tets if len(sc.tets) else None, tet_materials=sc.tet_materials,
                              hexes=sc.hexes if len(sc.hexes) else None, hex_materials=sc.hex_materials,
                              velocity=sc.velocity, radius=sc.radius, gravity=sc.gravity,
                              scene_offsets=scene_offsets, device=device)
    solver = SolverFEM(model, dt=sc.dt, solver_type="cg", preconditioner_type="block_diag",
                       linear_solver_maxiter=sc.maxiter, linear_solver_tolerance=sc.tolerance, self_contact_ke=0.0,
                       fixed_particle_indices=sc.fixed if len(sc.fixed) else None)
    return model, solver


def batched_measurement(device: str, steps: int, warmup: int) -> dict:
    """256 uneven scenes: one batched handle vs each scene stepped alone (both as captured frame graphs)."""
    import torch

    from newton_solver_fem_gb300 import scenes

    sc = scenes.batched_scenes()
    model, batched = scene_solver(sc, device, sc.scene_offsets)
    parts = [scene_solver(s, device) for s in scenes.split_batched(sc)]
    P = model.particle_count
    stream = torch.cuda.Stream(device)

    def frame(pairs):
        for mdl, slv, a, b in pairs:
            slv.refresh_tangent(a.particle_q)
            for _ in range(sc.substeps):
                slv.step(a, b, None, None, sc.dt)
                a, b = b, a

    runs = {
        "batched": [(model, batched, model.state(), model.state())],
        "plain": [(m, s, m.state(), m.state()) for m, s in parts],
    }
    out = {}
    for name, pairs in runs.items():
        with torch.cuda.stream(stream):
            frame(pairs)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream):
            with torch.cuda.graph(graph, stream=stream):
                frame(pairs)
        for _ in range(max(3, warmup)):
            graph.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(steps):
                graph.replay()
            e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        iters = [p[1].stats()["scene_iterations"] for p in pairs]
        flat = [i for it in iters for i in it]
        finite = all(bool(torch.isfinite(p[2].particle_q).all()) for p in pairs)
        out[name] = {"ms_per_frame": ms, "value": 3 * P * sc.substeps / (ms / 1e3), "unit": UNIT,
                     "mean_cg_iterations_last_substep": float(sum(flat) / len(flat)), "finite": finite}
        del graph
    out["scenes"] = len(sc.scene_offsets) - 1
    out["nodes"] = P
    out["speedup_batched_vs_plain"] = out["batched"]["value"] / out["plain"]["value"]
    out["workload"] = "256 scenes (128 Tet4, 128 Hex8), dims U{4..32}^3, cell 0.05 m, one face fixed, gravity"
    return out


def launch_shape(solver) -> dict:
    """The PCG launch configuration a handle uses (the tuning getters)."""
    import ctypes

    from newton_solver_fem_gb300 import _lib

    lib = _lib.load()
    out = {}
    for name, key in (("pcg_ctas", _lib.FEM_TUNE_GRID), ("cta_threads", _lib.FEM_TUNE_CTA_THREADS),
                      ("column_mode", _lib.FEM_TUNE_COMPACT_COLUMNS), ("l2_resident_slices", _lib.FEM_TUNE_RESIDENT_SLICES),
                      ("resident_row_state", _lib.FEM_TUNE_RESIDENT_STATE), ("spmv_unroll", _lib.FEM_TUNE_SPMV_UNROLL),
                      ("cg_variant", getattr(_lib, "FEM_TUNE_CG_VARIANT", None))):
        if key is None:
            continue
        v = ctypes.c_int64()
        _lib.check(lib.fem_get_tuning(solver._handle, key, ctypes.byref(v)))
        out[name] = int(v.value)
    return out


class FrameWindow:
    """Times K frames (tangent refresh + substeps, one captured CUDA graph each) starting from the
    workload's initial state: before the warm-up replays and again before the timed replays the
    state and the warm start are reset, so every run times the same simulated frames 0..K-1 whatever
    the warm-up count.  CG iterations over the timed frames come from the solver's counters."""

    def __init__(self, solver, model, substeps, dt, stream):
        import torch

        self.solver, self.substeps, self.dt, self.stream = solver, substeps, dt, stream
        self.a, self.b = model.state(), model.state()
        self.q0, self.v0 = self.a.particle_q.clone(), self.a.particle_qd.clone()
        with torch.cuda.stream(stream):
            self._frame()  # eager warm-up: first refresh, lazy setup
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream):
            with torch.cuda.graph(self.graph, stream=stream):
                self._frame()

    def _frame(self):
        x, y = self.a, self.b
        self.solver.refresh_tangent(x.particle_q)
        for _ in range(self.substeps):
            self.solver.step(x, y, None, None, self.dt)
            x, y = y, x
        if self.substeps % 2:  # keep the frame's result in state a
            self.a.particle_q.copy_(x.particle_q)
            self.a.particle_qd.copy_(x.particle_qd)

    def reset(self):
        import torch

        with torch.cuda.stream(self.stream):
            self.a.particle_q.copy_(self.q0)
            self.a.particle_qd.copy_(self.v0)
            self.solver.reset()
        torch.cuda.synchronize()

    def run(self, steps, warmup, clocks=None):
        """Returns (ms per frame, mean CG iterations per substep over the timed frames)."""
        import torch

        self.reset()
        for _ in range(max(3, warmup)):
            self.graph.replay()
        self.reset()
        it0 = self.solver.stats()["total_iterations"]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if clocks is not None:
            clocks.start()
        with torch.cuda.stream(self.stream):
            e0.record(self.stream)
            for _ in range(steps):
                self.graph.replay()
            e1.record(self.stream)
        torch.cuda.synchronize()
        clk = clocks.stop() if clocks is not None else None
        iters = (self.solver.stats()["total_iterations"] - it0) / (steps * self.substeps)
        return e0.elapsed_time(e1) / steps, iters, clk


def tet_measurement(device: str, steps: int, warmup: int) -> dict:
    """Jittered Tet4 48^3 block (663,552 tets, 795,024 edge springs, ground): frames 0..K-1 from the
    drop as captured graphs (the block lands on the ground at about frame 12)."""
    import torch

    from newton_solver_fem_gb300 import SolverFEM, model_from_arrays, scenes

    sc = scenes.tet_jittered_48()
    model = model_from_arrays(sc.x, sc.mass, tets=sc.tets, tet_materials=sc.tet_materials, springs=sc.springs,
                              spring_ke=sc.spring_ke, spring_kd=sc.spring_kd, velocity=sc.velocity,
                              radius=sc.radius, gravity=sc.gravity, device=device)
    ke, kd, kf, mu = sc.ground
    solver = SolverFEM(model, dt=sc.dt, solver_type="cg", preconditioner_type="block_diag",
                       linear_solver_maxiter=sc.maxiter, linear_solver_tolerance=sc.tolerance, self_contact_ke=0.0,
                       ground_plane=sc.ground_plane, ground_ke=ke, ground_kd=kd, ground_kf=kf, ground_mu=mu)
    P = model.particle_count
    window = FrameWindow(solver, model, sc.substeps, sc.dt, torch.cuda.Stream(device))
    ms, iters, _ = window.run(steps, warmup)
    finite = bool(torch.isfinite(window.a.particle_q).all())
    shape = launch_shape(solver)
    del window
    return {"workload": "tet4_jittered_48^3 (117,649 nodes, 663,552 tets, 795,024 springs, ground), "
                        f"10 substeps/frame, 50 CG at tol 1e-2, frames 0..{steps - 1} from the drop",
            "ms_per_frame": ms, "value": 3 * P * sc.substeps / (ms / 1e3), "unit": UNIT,
            "mean_cg_iterations": iters, "cg_iterations_timed": iters * steps * sc.substeps,
            "launch": shape, "l2_resident_matrix_bytes": 40 * solver.matrix_info()["stored_blocks"]
            if shape["l2_resident_slices"] else 0, "finite": finite}


def adjoint_measurement(device: str, repeats: int) -> dict:
    """Differentiable beam (16x4x4 cubes, 1,536 tets, 120 frames x 4 substeps, 30 CG): gradient vs plain rollout.

    Plain rollout: the 480 substeps through ``SolverFEM.step``, one captured
    graph per frame, replayed 120 times.  Gradient: the checkpointed gradient on
    the device (``adjoint.device_checkpointed_gradient``): the forward pass
    keeping a checkpoint every 10 frames, then per segment its recomputation and
    reverse pass replayed from one captured graph, plus the loss gradient in
    torch.  Both at the differentiable tolerance (1e-8, 30 CG iterations, every
    solve from zero).  The ratio is gradient time / plain time.
    """
    import torch

    from newton_solver_fem_gb300 import scenes
    from newton_solver_fem_gb300.adjoint import DeviceRollout, DifferentiableSolver, device_checkpointed_gradient

    sc = scenes.tet_beam()
    model, solver = scene_solver(sc, device)
    solver.linear_solver_tolerance = 1.0e-8
    P = model.particle_count
    steps = sc.frames * sc.substeps
    every = sc.extra["checkpoint_every"] * sc.substeps
    diff = DifferentiableSolver(solver, tolerance=1.0e-8, maxiter=sc.maxiter)
    scale = torch.tensor(sc.extra["mu_scale"], device=device)
    diff.set_mu_scale(scale)
    solver.refresh_tangent(model.particle_q.clone())
    tip = torch.as_tensor(sc.extra["tip_nodes"], device=device, dtype=torch.long)
    target = torch.tensor(sc.extra["target"], device=device, dtype=torch.float32)
    q0 = model.particle_q.clone()
    v0 = torch.zeros_like(q0)

    def loss_fn(q, v):
        return ((q[tip].mean(0) - target) ** 2).sum()

    def wall(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t, out

    a, b = model.state(), model.state()
    stream = torch.cuda.Stream(device)

    def plain_frame():
        x, y = a, b
        for _ in range(sc.substeps):
            solver.step(x, y, None, None, sc.dt)
            x, y = y, x

    with torch.cuda.stream(stream):
        plain_frame()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            plain_frame()

    def plain():
        with torch.cuda.stream(stream):
            for _ in range(sc.frames):
                graph.replay()

    # a second handle over the same beam recomputes each segment while the next one runs its reverse pass
    model2, solver2 = scene_solver(sc, device)
    solver2.linear_solver_tolerance = 1.0e-8
    solver2.refresh_tangent(model2.particle_q.clone())
    diff2 = DifferentiableSolver(solver2, tolerance=1.0e-8, maxiter=sc.maxiter)
    diff2.set_mu_scale(scale)
    rollout = DeviceRollout(diff, steps, every, overlap=diff2)

    def gradient():
        return device_checkpointed_gradient(diff, q0, v0, steps, every, loss_fn, mu_scale=scale, rollout=rollout)

    plain()
    gradient()  # warm-up: captures the segment graph
    res = {"plain_s": [], "gradient_s": []}
    for _ in range(max(1, repeats)):
        res["plain_s"].append(wall(plain)[0])
        t, (loss, g) = wall(gradient)
        res["gradient_s"].append(t)
    med = {k: float(sorted(v)[len(v) // 2]) for k, v in res.items()}
    dof_substeps = 3 * P * steps
    del graph
    return {
        "workload": "tet4_beam_16x4x4 hanging (425 nodes, 1,536 tets), 120 frames x 4 substeps, 30 CG at tol 1e-8, "
                    "loss on the tip-face centroid, gradients wrt 1,536 shear scales and v0, checkpoints every 10 "
                    "frames",
        "plain_ms": 1e3 * med["plain_s"], "plain_value": dof_substeps / med["plain_s"], "unit": UNIT,
        "checkpointed_gradient_ms": 1e3 * med["gradient_s"],
        "checkpointed_gradient_value": dof_substeps / med["gradient_s"],
        "gradient_over_plain": med["gradient_s"] / med["plain_s"],
        "recompute": "overlapped on a second handle and stream" if rollout.overlap is not None else "in line",
        "plain_cg_iterations_last_substep": solver.stats()["max_iterations"],
        "finite": bool(torch.isfinite(g["mu_scale"]).all()) and bool(torch.isfinite(loss))
                  and bool(torch.isfinite(a.particle_q).all()),
        "timer": "wall clock around synchronised passes, median of repeats", "repeats": max(1, repeats),
    }


def batched_adjoint_measurement(device: str, frames: int = 60) -> dict:
    """256 uneven scenes: a 60-frame rollout and its batched adjoint pass.

    Every frame refreshes the tangent at its start, as the frame loop does; a
    frame is one segment, whose matrix is fixed (the differentiable contract, no
    dA/dq), and its reverse pass reassembles the tangent at the frame's first
    state, so it uses the matrix the forward used.  The forward solves warm-start
    from the previous increment at the scenes' tolerance (1e-2, at most 50 CG),
    exactly like the plain path, and every substep's state is kept on the device
    (601 states x 1.56M nodes x 24 B = 22.5 GB of HBM), so nothing is recomputed;
    each adjoint solve warm-starts from the previous one.  The loss is the mean
    height of all nodes at the end; gradients are taken with respect to the
    initial velocities.  The plain rollout runs the same frames through
    ``SolverFEM.step``.
    """
    import torch

    from newton_solver_fem_gb300 import scenes
    from newton_solver_fem_gb300.adjoint import DeviceRollout, DifferentiableSolver, device_checkpointed_gradient

    sc = scenes.batched_scenes()
    model, solver = scene_solver(sc, device, sc.scene_offsets)
    P = model.particle_count
    steps = frames * sc.substeps
    diff = DifferentiableSolver(solver, tolerance=sc.tolerance, maxiter=sc.maxiter)
    q0, v0 = model.particle_q.clone(), model.particle_qd.clone()

    def loss_fn(q, v):
        return q[:, 2].mean()

    def plain():
        a, b = model.state(), model.state()
        a.particle_q.copy_(q0)
        a.particle_qd.copy_(v0)
        solver.reset()
        for _ in range(frames):
            solver.refresh_tangent(a.particle_q)
            for _ in range(sc.substeps):
                solver.step(a, b, None, None, sc.dt)
                a, b = b, a
        return a

    def wall(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t, out

    rollout = DeviceRollout(diff, steps, sc.substeps, refresh=True, warm_start=True, warm_adjoint=True,
                            store_all=True)

    def gradient():
        return device_checkpointed_gradient(diff, q0, v0, steps, sc.substeps, loss_fn, refresh=True,
                                            warm_start=True, warm_adjoint=True, store_all=True, rollout=rollout)

    wall(plain)  # warm-up
    t_plain, end = wall(plain)
    wall(gradient)
    t_grad, (loss, g) = wall(gradient)
    dv0 = g["v0"]
    return {"workload": "256 scenes (1.56M nodes), 60 frames x 10 substeps, tangent refreshed per frame, "
                        "tol 1e-2 / 50 CG, every substep state kept on the device, loss = mean node height, "
                        "gradient wrt v0",
            "plain_rollout_ms": 1e3 * t_plain, "gradient_ms": 1e3 * t_grad,
            "gradient_over_plain": t_grad / t_plain, "plain_value": 3 * P * steps / t_plain,
            "gradient_value": 3 * P * steps / t_grad, "unit": UNIT,
            "finite": bool(torch.isfinite(end.particle_q).all()) and bool(torch.isfinite(dv0).all())
                      and bool(torch.isfinite(loss)),
            "timer": "wall clock around synchronised passes"}


def run_gb300(args) -> None:
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    from newton_solver_fem_gb300 import _lib, build

    build.build()
    sc, model, solver, np = build_workload(args.cells, device)
    lib = _lib.load()
    P = model.particle_count
    info = solver.matrix_info()
    s0, s1 = model.state(), model.state()
    # the project's autotuner picks the PCG launch variant (staging depth, rows per CTA, CG recurrence)
    # on this workload, timing each candidate's launches from the same initial state
    from newton_solver_fem_gb300 import autotune

    q_start, v_start = model.particle_q.clone(), model.particle_qd.clone()

    def tune_restore():
        s0.particle_q.copy_(q_start)
        s0.particle_qd.copy_(v_start)
        solver.reset()

    def tune_frame():
        a, b = s0, s1
        solver.refresh_tangent(a.particle_q)
        for _ in range(sc.substeps):
            solver.step(a, b, None, None, sc.dt)
            a, b = b, a

    tuned = autotune.autotune(solver, tune_frame, tune_restore, frames=2, use_cache=False)
    tune_restore()
    # then split the PCG rows over the CTAs by their measured SpMV speed (a public tuning key;
    # about 1% on this workload, deterministic for the handle)
    _lib.check(lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_BALANCE, 1))
    substeps = sc.substeps
    stream = torch.cuda.Stream(device)

    def frame(a, b):
        solver.refresh_tangent(a.particle_q)
        for k in range(substeps):
            solver.step(a, b, None, None, sc.dt)
            a, b = b, a

    with torch.cuda.stream(stream):
        if args.trace_iterations:
            a, b = s0, s1
            solver.refresh_tangent(a.particle_q)
            for k in range(substeps):
                solver.step(a, b, None, None, sc.dt)
                a, b = b, a
                torch.cuda.synchronize()
                print(json.dumps({"pcg_launch": k, "iterations": solver.stats()["max_iterations"]}), file=sys.stderr,
                      flush=True)
        else:
            frame(s0, s1)  # eager warm-up (first refresh, lazy setup)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            frame(s0, s1)
    q_init, v_init = model.particle_q.clone(), model.particle_qd.clone()

    def reset_state():
        """Frames 0..K-1 from the workload's initial state, whatever the warm-up count."""
        with torch.cuda.stream(stream):
            s0.particle_q.copy_(q_init)
            s0.particle_qd.copy_(v_init)
            solver.reset()
        torch.cuda.synchronize()

    reset_state()
    for _ in range(max(3, args.warmup)):
        graph.replay()
    reset_state()
    if world > 1:
        torch.distributed.barrier()
    it_timed0 = solver.stats()["total_iterations"]
    clocks = ClockSampler(local)
    clocks.start()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        start.record(stream)
        for _ in range(args.steps):
            graph.replay()
        end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = start.elapsed_time(end) / args.steps
    timed_iterations = (solver.stats()["total_iterations"] - it_timed0) / (args.steps * substeps)
    from newton_solver_fem_gb300.replicas import max_over_ranks

    ms = max_over_ranks(ms, device)  # replicas: the slowest rank sets the job time
    value = world * 3 * P * substeps / (ms / 1e3)

    # ---- roofline of the dominant kernel: eager frames (0..2 from the initial state) with per-launch CUDA events
    reset_state()
    stats0 = solver.stats()
    _lib.check(lib.fem_set_timing(solver._handle, 1))
    with torch.cuda.stream(stream):
        for _ in range(max(1, min(args.steps, 3))):
            frame(s0, s1)
    total_ms, launches = torch.tensor(0.0), 0
    import ctypes

    t_ms, n_l = ctypes.c_double(), ctypes.c_int64()
    _lib.check(lib.fem_get_timing(solver._handle, ctypes.byref(t_ms), ctypes.byref(n_l)))
    _lib.check(lib.fem_set_timing(solver._handle, 0))
    stats1 = solver.stats()
    launches = n_l.value
    iters = (stats1["total_iterations"] - stats0["total_iterations"]) / max(1, launches)
    launch_ms = t_ms.value / max(1, launches)
    cc = ctypes.c_int64()
    _lib.check(lib.fem_get_tuning(solver._handle, _lib.FEM_TUNE_COMPACT_COLUMNS, ctypes.byref(cc)))
    ub = ctypes.c_int64()
    _lib.check(lib.fem_get_tuning(solver._handle, _lib.FEM_TUNE_UNIFORM_COLUMN_BLOCKS, ctypes.byref(ub)))
    # column bytes read per stored block: 32-bit columns, 16-bit offsets, or 16-bit offsets only outside
    # the slots whose offset is shared by the slice (read once per slice: 8 B mask + 2 B per slot)
    col_bytes = 4.0 if cc.value == 0 else 2.0 * (info["nnzb"] - ub.value) / info["nnzb"]
    bytes_launch = pcg_launch_bytes(info["nnzb"], P, iters, col_bytes)
    achieved = bytes_launch / (launch_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic = dram_traffic_per_launch(iters) if args.cells == 64 else None

    op_tuned = autotune.tune_operator(solver)  # standalone SpMV: loads in flight, or bulk-copy staging
    spmv = standalone_spmv(solver, lib, P, info["nnzb"], peak)
    spmv["operator_tuning"] = op_tuned

    # ---- end to end through the public API with host buffers, driven the way the reference's own
    # example drives its solver (examples/example_linear_fem.py:107-128): per frame an eager tangent
    # refresh, then a captured CUDA graph of the substeps' SolverFEM.step calls
    host_q = torch.empty((P, 3), dtype=torch.float32, pin_memory=True)
    host_v = torch.empty((P, 3), dtype=torch.float32, pin_memory=True)
    e2e_steps = max(1, args.steps)

    def substeps_only(a, b):
        for _ in range(substeps):
            solver.step(a, b, None, None, sc.dt)
            a, b = b, a

    substep_graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(substep_graph, stream=stream):
            substeps_only(s0, s1)

    def e2e_frames(count):
        with torch.cuda.stream(stream):
            for _ in range(count):
                s0.particle_q.copy_(host_q, non_blocking=True)
                s0.particle_qd.copy_(host_v, non_blocking=True)
                solver.refresh_tangent(s0.particle_q)
                substep_graph.replay()
                host_q.copy_(s0.particle_q, non_blocking=True)
                host_v.copy_(s0.particle_qd, non_blocking=True)
            stream.synchronize()

    # untimed warm-up through the same calls, then frames 0..K-1 from the initial state like the timed window
    for warm in (True, False):
        host_q.copy_(q_init.cpu())
        host_v.copy_(v_init.cpu())
        reset_state()
        if warm:
            e2e_frames(max(3, args.warmup))
    t0 = time.perf_counter()
    e2e_frames(e2e_steps)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_value = world * 3 * P * substeps / e2e_s
    finite = bool(torch.isfinite(s0.particle_q).all())
    batched = None
    if not args.no_batched and rank == 0:
        batched = batched_measurement(device, args.steps, args.warmup)
    adjoint = None
    if not args.no_adjoint and rank == 0:
        adjoint = adjoint_measurement(device, 3)
    tet = None
    if not args.no_tet and rank == 0:
        tet = tet_measurement(device, args.steps, args.warmup)
    if batched is not None and not args.no_adjoint:
        batched["adjoint"] = batched_adjoint_measurement(device)

    if rank == 0:
        cpu = None if args.no_cpu_baseline else cpu_baseline(args.cpu_cells or args.cells, args.cpu_sample)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"hex8_block_{args.cells}^3", "nodes": P, "hexes": int(model.fem.hex_count),
                       "dof": 3 * P, "substeps_per_step": substeps, "cg_tol": sc.tolerance,
                       "cg_maxiter": sc.maxiter, "preconditioner": "block_diag", "parallelism": "replicas",
                       "nnzb": info["nnzb"], "mean_cg_iterations": timed_iterations,
                       "frames": f"0..{args.steps - 1} from the initial state (reset after warm-up)",
                       "autotuned": {"choice": {k: tuned[k] for k in ("unroll", "threads", "cg_variant", "grid")},
                                     "us_per_cg_iteration": {
                                         f"u{r['unroll']}_t{r['threads']}_v{r['cg_variant']}":
                                             round(r["us_per_iteration"], 2) for r in tuned["candidates"]}},
                       "launch": launch_shape(solver),
                       "pcg_split": "rows split over CTAs by calibrated SpMV speed (FEM_TUNE_BALANCE=1)",
                       "column_mode": int(cc.value), "column_index_bytes": round(col_bytes, 4),
                       "l2": "inputs larger than L2 (A values 259 MB, element blocks 614 MB at 64^3)"},
            "roofline": {"kernel": "pcg_kernel", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of two full 64^3 launches "
                                           "(18 and 22 CG iterations), linear in the iteration count, at this run's "
                                           "mean (profiles/pcg_kernel_hex8_64_dram.md)" if traffic else None,
                         "bytes_per_launch": bytes_launch, "launch_ms": launch_ms, "launches": launches},
            "spmv": spmv,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * 12 * P,
                    "d2h_bytes_per_step": 2 * 12 * P,
                    "calls": "per frame: pinned H2D of q and v, SolverFEM.refresh_tangent, replay of a captured "
                             f"graph of {substeps} SolverFEM.step calls, D2H of q and v; wall clock"},
            "gpu_launches": args.steps * (3 + 4 * substeps),
            "clocks": clk,
            "cpu_baseline": cpu,
            "finite": finite,
            "batched": batched,
            "adjoint": adjoint,
            "tet": tet,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def standalone_spmv(solver, lib, P: int, nnzb: int, peak: float) -> dict:
    """One (PAP + I - P) x through the public fem_apply_operator, timed alone (CUDA events on the
    launching stream, median of 30 launches).  Before each launch a 512 MB buffer is written and then a
    second 512 MB buffer is read: the read evicts the first buffer's dirty lines, so the timed launch
    starts with an L2 of clean lines that are not the matrix's, and pays for no write-back of the flush."""
    import ctypes

    import torch

    from newton_solver_fem_gb300 import _lib

    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn((P, 3), device="cuda", generator=g)
    y = torch.empty_like(x)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    clean = torch.ones(128 << 20, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    cc = ctypes.c_int64()
    _lib.check(lib.fem_get_tuning(solver._handle, _lib.FEM_TUNE_COMPACT_COLUMNS, ctypes.byref(cc)))
    times = []
    for _ in range(31):
        flush.fill_(1)
        clean.sum()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _lib.check(lib.fem_apply_operator(solver._handle, x.data_ptr(), y.data_ptr(), stream.cuda_stream))
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    us = 1e3 * statistics.median(times[1:])
    col = 4 if cc.value == 0 else 2  # the operator reads 16-bit offsets whenever the handle has them
    gbs = spmv_bytes(nnzb, P, col) / (us / 1e6) / 1e9
    stage, batch = ctypes.c_int64(), ctypes.c_int64()
    _lib.check(lib.fem_get_tuning(solver._handle, _lib.FEM_TUNE_OPERATOR_STAGE, ctypes.byref(stage)))
    _lib.check(lib.fem_get_tuning(solver._handle, _lib.FEM_TUNE_OPERATOR_BATCH, ctypes.byref(batch)))
    kernel = (f"apply_operator_staged_kernel<{stage.value}> (fem_apply_operator, bulk-copy staging)"
              if stage.value and col == 2 else f"apply_operator_kernel<{batch.value}> (fem_apply_operator)")
    return {"kernel": kernel, "us": us, "achieved": gbs, "peak": peak,
            "unit": "GB/s", "frac": gbs / peak, "column_index_bytes": col}


def profile_workload(name: str, steps: int, cells: int = 64) -> None:
    """Eager frames (tangent refresh + substeps) of one workload, for profiling; prints the CG
    iterations of every PCG launch in launch order (maps an ncu launch index to its iteration count)."""
    import torch

    from newton_solver_fem_gb300 import scenes

    if name == "hex":
        sc, model, solver, _ = build_workload(cells, "cuda:0")
    elif name == "batched":
        sc = scenes.batched_scenes()
        model, solver = scene_solver(sc, "cuda:0", sc.scene_offsets)
    else:
        from newton_solver_fem_gb300 import SolverFEM, model_from_arrays

        sc = scenes.tet_jittered_48()
        model = model_from_arrays(sc.x, sc.mass, tets=sc.tets, tet_materials=sc.tet_materials, springs=sc.springs,
                                  spring_ke=sc.spring_ke, spring_kd=sc.spring_kd, velocity=sc.velocity,
                                  radius=sc.radius, gravity=sc.gravity, device="cuda:0")
        ke, kd, kf, mu = sc.ground
        solver = SolverFEM(model, dt=sc.dt, solver_type="cg", preconditioner_type="block_diag",
                           linear_solver_maxiter=sc.maxiter, linear_solver_tolerance=sc.tolerance,
                           self_contact_ke=0.0, ground_plane=sc.ground_plane, ground_ke=ke, ground_kd=kd,
                           ground_kf=kf, ground_mu=mu)
    a, b = model.state(), model.state()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    iterations = []
    for _ in range(steps):
        solver.refresh_tangent(a.particle_q)
        for _ in range(sc.substeps):
            solver.step(a, b, None, None, sc.dt)
            iterations.append(solver.stats()["max_iterations"])  # synchronises: launch order is preserved
            a, b = b, a
    e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"pcg_launch_iterations": iterations}), file=sys.stderr)
    print(f"{name}: {steps} eager frames, {e0.elapsed_time(e1) / max(1, steps):.3f} ms per frame, "
          f"{model.particle_count} nodes, last substep max CG iterations {solver.stats()['max_iterations']}",
          file=sys.stderr)


def main():
    args = parse()
    if args.profile_workload is not None:
        profile_workload(args.profile_workload, args.steps, args.cells)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
