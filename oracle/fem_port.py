"""TEST INFRASTRUCTURE ONLY: driver of the C/OpenMP CPU port (``oracle/fem_port.c``).

Used as the timed CPU baseline (``bench.py`` cpu_baseline leg and
``--impl reference``) and checked against the NumPy oracle by
``tests/test_port.py``.  Setup (pattern, slot lists, incidence lists) is done
here with NumPy; every per-frame and per-substep pass runs in C with OpenMP on
all host cores.  Build with ``make -C oracle`` (or ``build_port()``).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

from oracle import fem_oracle as O

HERE = Path(__file__).resolve().parent
LIBRARY = HERE / "_build" / "libfemport.so"


def build_port() -> Path:
    """Compile the port with gcc -O3 -fopenmp (portable flags, no -march)."""
    src = HERE / "fem_port.c"
    LIBRARY.parent.mkdir(exist_ok=True)
    if not LIBRARY.exists() or LIBRARY.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIBRARY


_LIB = None


def load():
    global _LIB
    if _LIB is None:
        build_port()
        lib = ctypes.CDLL(str(LIBRARY))
        p, i64, f = ctypes.c_void_p, ctypes.c_int64, ctypes.c_float
        lib.port_threads.restype = ctypes.c_int
        lib.port_tet_forces.argtypes = [i64, p, p, p, p, p, f, f, p]
        lib.port_hex_forces.argtypes = [i64, p, p, p, p, p, p, f, f, p]
        lib.port_spring_forces.argtypes = [i64, p, p, p, p, p, p, p]
        lib.port_tet_tangent.argtypes = [i64, p, p, p, p, f, f, f, p]
        lib.port_hex_tangent.argtypes = [i64, p, p, p, p, p, f, f, f, p]
        lib.port_gather.argtypes = [i64, p, p, p, p]
        lib.port_node_gather.argtypes = [i64, p, p, p, p]
        lib.port_block_jacobi.argtypes = [i64, p, p, p, p]
        lib.port_solve.argtypes = [i64, p, p, p, p, p, p, p, p, p, p, p, p, f, f, ctypes.c_int, p]
        lib.port_solve.restype = ctypes.c_int
        _LIB = lib
    return _LIB


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def _csr(keys: np.ndarray, n: int):
    """Entries grouped by key (stable, ascending entry id) -> (ptr [n+1], ent)."""
    order = np.argsort(keys, kind="stable").astype(np.int32)
    ptr = np.zeros(n + 1, np.int64)
    np.add.at(ptr, keys + 1, 1)
    return np.cumsum(ptr).astype(np.int32), order


class PortFEM:
    """Float32 CPU port of the hot path for one scene (Tet4 and/or Hex8, springs, ground, gravity, fixed nodes)."""

    def __init__(self, x, mass, *, tets=None, tet_poses=None, tet_materials=None, hexes=None, hex_inv_J0=None,
                 hex_det_J0_w=None, hex_materials=None, springs=None, spring_rest=None, spring_ke=None, spring_kd=None,
                 gravity=(0.0, 0.0, -9.81), dt=1.0 / 600.0, min_stretch=0.05,
                 max_stretch=20.0, ground_plane=None, ground=(1.0e5, 1.0e2, 1.0e3, 0.5), radius=0.0, fixed=None,
                 maxiter=50, tolerance=1.0e-2):
        self.lib = load()
        f32 = np.float32
        self.rest = np.ascontiguousarray(x, f32)
        self.n = n = len(self.rest)
        self.mass = np.ascontiguousarray(mass, f32)
        self.inv_mass = np.where(self.mass > 0, 1.0 / np.where(self.mass > 0, self.mass, 1), 0).astype(f32)
        self.tets = np.ascontiguousarray(np.zeros((0, 4)) if tets is None else tets, np.int32)
        self.tet_poses = np.ascontiguousarray(np.zeros((0, 3, 3)) if tet_poses is None else tet_poses, f32)
        self.tet_mat = np.ascontiguousarray(np.zeros((0, 3)) if tet_materials is None else tet_materials, f32)
        self.hexes = np.ascontiguousarray(np.zeros((0, 8)) if hexes is None else hexes, np.int32)
        self.hex_invJ = np.ascontiguousarray(np.zeros((0, 8, 3, 3)) if hex_inv_J0 is None else hex_inv_J0, f32)
        self.hex_detw = np.ascontiguousarray(np.zeros((0, 8)) if hex_det_J0_w is None else hex_det_J0_w, f32)
        self.hex_mat = np.ascontiguousarray(np.zeros((0, 3)) if hex_materials is None else hex_materials, f32)
        self.gravity = np.asarray(gravity, np.float64)
        self.dt, self.lo, self.hi = float(dt), float(min_stretch), float(max_stretch)
        self.ground_plane = None if ground_plane is None else np.asarray(ground_plane, np.float64)
        self.ground = ground
        self.radius = np.broadcast_to(np.asarray(radius, np.float64), (n,))
        self.fixed = np.zeros(0, np.int64) if fixed is None else np.unique(np.asarray(fixed, np.int64))
        self.fixed_mask = np.zeros(n, np.uint8)
        self.fixed_mask[self.fixed] = 1
        self.maxiter, self.tol = int(maxiter), float(tolerance)
        self.springs = np.ascontiguousarray(np.zeros((0, 2)) if springs is None else springs, np.int32)
        S = len(self.springs)
        rest_len = np.linalg.norm(self.rest[self.springs[:, 0]] - self.rest[self.springs[:, 1]], axis=1) \
            if spring_rest is None else spring_rest
        self.spring_rest = np.ascontiguousarray(rest_len, f32)
        self.spring_ke = np.ascontiguousarray(np.zeros(S) if spring_ke is None else spring_ke, f32)
        self.spring_kd = np.ascontiguousarray(np.zeros(S) if spring_kd is None else spring_kd, f32)
        T, H = len(self.tets), len(self.hexes)
        # triplet layout [P | 2S | 16T | 64H] (solver.py:312-321; springs as (a, b), (b, a) pairs)
        sp_rows = self.springs.reshape(-1)
        sp_cols = self.springs[:, ::-1].reshape(-1)
        rows = np.concatenate([np.arange(n), sp_rows, np.repeat(self.tets, 4, axis=1).ravel(),
                               np.repeat(self.hexes, 8, axis=1).ravel()])
        cols = np.concatenate([np.arange(n), sp_cols, np.tile(self.tets, (1, 4)).ravel(),
                               np.tile(self.hexes, (1, 8)).ravel()])
        valid = (rows >= 0) & (cols >= 0)  # springs with a negative index add no block
        rows, cols = np.where(valid, rows, 0), np.where(valid, cols, 0)
        key = np.where(valid, rows.astype(np.int64) * n + cols, -1)
        order = np.argsort(key, kind="stable")
        order = order[key[order] >= 0]
        ks = key[order]
        uniq, start = np.unique(ks, return_index=True)
        self.contrib = order.astype(np.int32)
        self.cptr = np.append(start, len(ks)).astype(np.int32)
        r = (uniq // n).astype(np.int64)
        self.columns = (uniq % n).astype(np.int32)
        off = np.zeros(n + 1, np.int64)
        np.add.at(off, r + 1, 1)
        self.offsets = np.cumsum(off).astype(np.int32)
        self.nnzb = len(uniq)
        self.trip = np.zeros((len(rows), 9), f32)
        self.values = np.zeros((self.nnzb, 9), f32)
        self.minv = np.zeros((n, 9), f32)
        self.elem_tet = np.zeros((4 * T, 3), f32)
        self.elem_hex = np.zeros((8 * H, 3), f32)
        self.elem_spring = np.zeros((2 * S, 3), f32)
        ends = self.springs.reshape(-1).astype(np.int64)
        self.spring_ptr, self.spring_ent = _csr(np.where(ends >= 0, ends, n), n + 1)
        self.tet_ptr, self.tet_ent = _csr(self.tets.ravel().astype(np.int64), n)
        self.hex_ptr, self.hex_ent = _csr(self.hexes.ravel().astype(np.int64), n)
        self.dv = np.zeros((n, 3), f32)
        self.work = np.zeros(15 * n, f32)
        self._set_constant(self.dt)
        self.refresh_tangent(self.rest)

    def _set_constant(self, dt):
        """Mass + spring (h d + h^2 k) diagonal and -(h d + h^2 k) I off-diagonal blocks (solver.py:1015-1060)."""
        n, S = self.n, len(self.springs)
        h = np.float32(dt)
        c = (h * self.spring_kd + h * h * self.spring_ke).astype(np.float32)
        diag = self.mass.astype(np.float32).copy()
        for col in (0, 1):
            idx = self.springs[:, col]
            ok = idx >= 0
            np.add.at(diag, idx[ok], c[ok])
        d = np.zeros((n, 9), np.float32)
        d[:, 0] = d[:, 4] = d[:, 8] = diag
        self.trip[:n] = d
        if S:
            off = np.zeros((2 * S, 9), np.float32)
            cc = np.repeat(-c, 2)
            off[:, 0] = off[:, 4] = off[:, 8] = cc
            self.trip[n:n + 2 * S] = off

    def refresh_tangent(self, q):
        q = np.ascontiguousarray(q, np.float32).copy()
        q[self.fixed] = self.rest[self.fixed]
        n, T, H, L = self.n, len(self.tets), len(self.hexes), self.lib
        base = n + 2 * len(self.springs)
        if T:
            L.port_tet_tangent(T, _p(self.tets), _p(self.tet_poses), _p(self.tet_mat), _p(q), self.lo, self.hi, self.dt,
                               _p(self.trip[base:]))
        if H:
            L.port_hex_tangent(H, _p(self.hexes), _p(self.hex_invJ), _p(self.hex_detw), _p(self.hex_mat), _p(q),
                               self.lo, self.hi, self.dt, _p(self.trip[base + 16 * T:]))
        L.port_gather(self.nnzb, _p(self.cptr), _p(self.contrib), _p(self.trip), _p(self.values))
        L.port_block_jacobi(n, _p(self.offsets), _p(self.columns), _p(self.values), _p(self.minv))
        return q

    def step(self, q, v, dt):
        q = np.ascontiguousarray(q, np.float32).copy()
        v = np.ascontiguousarray(v, np.float32).copy()
        q[self.fixed] = self.rest[self.fixed]
        v[self.fixed] = 0.0
        n, T, H, L = self.n, len(self.tets), len(self.hexes), self.lib
        ft = np.zeros((n, 3), np.float32)
        fh = np.zeros((n, 3), np.float32)
        fs = np.zeros((n + 1, 3), np.float32)
        S = len(self.springs)
        if S:
            L.port_spring_forces(S, _p(self.springs), _p(self.spring_rest), _p(self.spring_ke), _p(self.spring_kd),
                                 _p(q), _p(v), _p(self.elem_spring))
            L.port_node_gather(n, _p(self.spring_ptr), _p(self.spring_ent), _p(self.elem_spring), _p(fs))
        if T:
            L.port_tet_forces(T, _p(self.tets), _p(self.tet_poses), _p(self.tet_mat), _p(q), _p(v), self.lo, self.hi,
                              _p(self.elem_tet))
            L.port_node_gather(n, _p(self.tet_ptr), _p(self.tet_ent), _p(self.elem_tet), _p(ft))
        if H:
            L.port_hex_forces(H, _p(self.hexes), _p(self.hex_invJ), _p(self.hex_detw), _p(self.hex_mat), _p(q), _p(v),
                              self.lo, self.hi, _p(self.elem_hex))
            L.port_node_gather(n, _p(self.hex_ptr), _p(self.hex_ent), _p(self.elem_hex), _p(fh))
        h = np.float32(dt)
        f = fs[:n] * h + ft * h + fh * h  # term order: spring, tet, hex (solver.py:571-582)
        if self.ground_plane is not None:
            ke, kd, kf, mu = self.ground
            fg = O.ground_forces(q, v, self.radius, self.inv_mass, np.ones(n, np.int32), ke, kd, kf, mu,
                                 self.ground_plane, self.gravity)
            f = f + fg.astype(np.float32) * h
        f = f + (np.outer(self.mass, self.gravity).astype(np.float32)) * h
        if S:  # spring damping restored after the elastic predictor (implicit_predictor.py:26-41); rhs = f - cv
            a, b = self.springs[:, 0], self.springs[:, 1]
            ok = (a >= 0) & (b >= 0)
            corr = (h * self.spring_kd[ok, None]) * (v[a[ok]] - v[b[ok]])
            np.add.at(f, a[ok], corr)
            np.subtract.at(f, b[ok], corr)
        f = np.ascontiguousarray(f, np.float32)
        q_out = np.empty_like(q)
        v_out = np.empty_like(v)
        it = L.port_solve(n, _p(self.offsets), _p(self.columns), _p(self.values), _p(self.minv), _p(self.fixed_mask),
                          _p(self.rest), _p(q), _p(v), _p(f), _p(self.dv), _p(q_out), _p(v_out), dt, self.tol,
                          self.maxiter, _p(self.work))
        self.last_iterations = it
        return q_out, v_out, f


def threads() -> int:
    return int(load().port_threads())


if __name__ == "__main__":
    build_port()
    print(LIBRARY, os.cpu_count(), threads())
