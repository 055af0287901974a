"""Autotuner selection and cache logic on CPU, with the GPU measurement replaced by a fake."""

import json

from newton_solver_fem_gb300 import _lib, autotune


class FakeSolver:
    device = "cpu"

    def __init__(self):
        self.applied = []


def _sig(choice):
    return tuple(choice[k] for k in ("unroll", "threads", "cg_variant"))


def _patch(monkeypatch, tmp_path, timings):
    monkeypatch.setattr(autotune, "CACHE", tmp_path / "tune.json")
    monkeypatch.setattr(autotune, "_key", lambda solver: "fake-gpu|P=8")
    monkeypatch.setattr(autotune, "apply", lambda solver, choice: solver.applied.append(dict(choice)))
    monkeypatch.setattr(autotune, "current", lambda solver: dict(solver.applied[-1]))
    monkeypatch.setattr(autotune, "measure", lambda solver, frame, restore, frames:
                        {"us_per_iteration": timings[_sig(solver.applied[-1])], "launch_ms": 1.0, "iterations": 9.0})


def _cand(u, t, v=0):
    return dict(unroll=u, threads=t, cg_variant=v, resident_bytes=-2)


def test_picks_fastest_and_applies_it(monkeypatch, tmp_path):
    cands = [_cand(4, 1024), _cand(2, 1024), _cand(4, 256), _cand(4, 1024, 1)]
    timings = {(4, 1024, 0): 75.0, (2, 1024, 0): 74.0, (4, 256, 0): 80.0, (4, 1024, 1): 76.0}
    _patch(monkeypatch, tmp_path, timings)
    s = FakeSolver()
    best = autotune.autotune(s, None, None, candidates=cands, use_cache=False)
    assert _sig(best) == (2, 1024, 0)
    assert _sig(s.applied[-1]) == (2, 1024, 0)
    assert [_sig(c) for c in s.applied[:4]] == [_sig(c) for c in cands]
    assert len(best["candidates"]) == 4


def test_cache_round_trip_skips_measurement(monkeypatch, tmp_path):
    cands = [_cand(4, 1024), _cand(4, 512)]
    _patch(monkeypatch, tmp_path, {(4, 1024, 0): 70.0, (4, 512, 0): 72.0})
    first = autotune.autotune(FakeSolver(), None, None, candidates=cands)
    assert json.loads((tmp_path / "tune.json").read_text())["fake-gpu|P=8"]["threads"] == 1024
    monkeypatch.setattr(autotune, "measure", lambda *a: (_ for _ in ()).throw(AssertionError("measured again")))
    s = FakeSolver()
    again = autotune.autotune(s, None, None, candidates=cands)
    assert again == first and _sig(s.applied[0]) == (4, 1024, 0)


def test_default_candidates_cover_every_axis():
    c = autotune.DEFAULT_CANDIDATES
    assert {x["threads"] for x in c} == {256, 512, 1024}  # rows per CTA
    assert {x["unroll"] for x in c} == {1, 2, 4}  # staging depth
    assert {x["cg_variant"] for x in c} == {0, 1}  # the CG recurrence
    assert all(x["resident_bytes"] == -2 for x in c)  # automatic L2 residency
    assert set(autotune.AXES.values()) >= {_lib.FEM_TUNE_SPMV_UNROLL, _lib.FEM_TUNE_CTA_THREADS,
                                           _lib.FEM_TUNE_CG_VARIANT}


def test_operator_search_covers_batch_and_bulk_staging_and_applies_the_faster(monkeypatch):
    state = {}

    class Lib:
        def fem_set_tuning(self, handle, key, value):
            state[key] = value
            return 0

    monkeypatch.setattr(_lib, "load", lambda: Lib())

    class S:
        _handle = None

    times = {(2, 0): 51.0, (4, 0): 63.0, (2, 4): 49.0, (2, 8): 55.0}
    timer = lambda solver: times[(state[_lib.FEM_TUNE_OPERATOR_BATCH], state[_lib.FEM_TUNE_OPERATOR_STAGE])]
    out = autotune.tune_operator(S(), timer=timer)
    assert (out["operator_batch"], out["operator_stage"]) == (2, 4)
    assert (state[_lib.FEM_TUNE_OPERATOR_BATCH], state[_lib.FEM_TUNE_OPERATOR_STAGE]) == (2, 4)
    assert {(r["operator_batch"], r["operator_stage"]) for r in out["candidates"]} == set(times)
