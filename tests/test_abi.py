"""The C-ABI library loads and exports every symbol ``include/fem_gb300.h`` declares (no GPU calls)."""

import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from newton_solver_fem_gb300 import _lib, build

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "fem_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(fem_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def library():
    build.build()
    return _lib.load()


def test_header_declares_the_reference_boundary():
    names = declared_functions()
    for required in ("fem_create", "fem_destroy", "fem_step", "fem_refresh_tangent", "fem_set_tolerance",
                     "fem_get_stats", "fem_export_bsr"):
        assert required in names


def test_every_declared_symbol_is_exported_and_bound(library):
    names = declared_functions()
    bound = {name for name, _, _ in _lib.SIGNATURES}
    for name in names:
        assert hasattr(library, name), name
        assert name in bound, f"{name} missing from _lib.SIGNATURES"
    assert library.fem_version().decode().startswith("fem_gb300")


def test_ctypes_struct_layout_matches_c(tmp_path):
    """sizeof/offsetof of FemDesc, FemStats and FemPreparedWs as gcc lays them out equal the ctypes mirrors."""
    fields = [name for name, _ in _lib.FemDesc._fields_]
    ws_fields = [name for name, _ in _lib.FemPreparedWs._fields_]
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void) {",
             'printf("%zu %zu %zu\\n", sizeof(FemDesc), sizeof(FemStats), sizeof(FemPreparedWs));']
    lines += [f'printf("%zu\\n", offsetof(FemPreparedWs, {f}));' for f in ws_fields]
    lines += [f'printf("%zu\\n", offsetof(FemDesc, {f}));' for f in fields]
    lines += ["return 0; }"]
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert int(out[0]) == ctypes.sizeof(_lib.FemDesc)
    assert int(out[1]) == ctypes.sizeof(_lib.FemStats)
    assert int(out[2]) == ctypes.sizeof(_lib.FemPreparedWs)
    for f, off in zip(ws_fields, out[3:3 + len(ws_fields)]):
        assert getattr(_lib.FemPreparedWs, f).offset == int(off), f
    for f, off in zip(fields, out[3 + len(ws_fields):]):
        assert getattr(_lib.FemDesc, f).offset == int(off), f


def test_bad_arguments_are_rejected_without_a_gpu(library):
    """Argument validation happens on the host before any device call."""
    d = _lib.FemDesc()
    d.particle_count = 4
    d.tolerance = 0.0  # invalid
    h = ctypes.c_void_p()
    code = library.fem_create(ctypes.byref(d), ctypes.byref(h))
    assert code == _lib.FEM_ERR_BAD_ARG
    assert library.fem_create(None, ctypes.byref(h)) == _lib.FEM_ERR_BAD_ARG
    with pytest.raises(ValueError):
        _lib.check(code)


def _message(library, code):
    return library.fem_status_string(code).decode()


def test_every_rejection_reports_its_own_message(library):
    """Each entry point names itself in the status message of a host-side rejection, so
    a message left over from an earlier call is never reported instead."""
    ws = _lib.FemPreparedWs()
    cases = [
        ("fem_prepare", lambda: library.fem_prepare(None, ctypes.byref(ws), None, None, None, None, None, 0.01, None)),
        ("fem_prepared_rhs", lambda: library.fem_prepared_rhs(None, ctypes.byref(ws), None, 0.01, None, None)),
        ("fem_apply_operator", lambda: library.fem_apply_operator(None, None, None, None)),
        ("fem_apply_preconditioner", lambda: library.fem_apply_preconditioner(None, None, None, None)),
        ("fem_prepared_solve",
         lambda: library.fem_prepared_solve(None, ctypes.byref(ws), None, 1e-6, 10, 0.01, None)),
        ("fem_prepared_reconstruct",
         lambda: library.fem_prepared_reconstruct(None, ctypes.byref(ws), None, 0.01, None, None, None)),
        ("fem_set_mu_scale", lambda: library.fem_set_mu_scale(None, None)),
        ("fem_solve", lambda: library.fem_solve(None, None, None, 1e-6, 10, None)),
        ("fem_force_vjp", lambda: library.fem_force_vjp(*([None] * 11))),
        ("fem_predictor_vjp", lambda: library.fem_predictor_vjp(None, None, 0.01, None, None)),
        ("fem_pcg_solve_noalloc",
         lambda: library.fem_pcg_solve_noalloc(None, None, None, None, None, 4, 1e-6, 10, None, None)),
        ("rows outside", lambda: library.fem_pcg_solve_noalloc(None, None, None, None, None, -1, 1e-6, 10, None, None)),
        ("tolerance", lambda: library.fem_pcg_solve_noalloc(None, None, None, None, None, 4, 0.0, 10, None, None)),
    ]
    for expected, call in cases:
        assert library.fem_create(None, None) == _lib.FEM_ERR_BAD_ARG  # leaves a different message behind
        code = call()
        assert code == _lib.FEM_ERR_BAD_ARG, expected
        assert expected in _message(library, code), (expected, _message(library, code))
