"""Autotuner selection and cache logic on CPU, with the GPU measurement replaced by a fake."""

import json

from newton_solver_fem_gb300 import autotune


class FakeSolver:
    device = "cpu"

    def __init__(self):
        self.applied = []


def _patch(monkeypatch, tmp_path, timings):
    monkeypatch.setattr(autotune, "CACHE", tmp_path / "tune.json")
    monkeypatch.setattr(autotune, "_key", lambda solver: "fake-gpu|P=8")
    monkeypatch.setattr(autotune, "apply", lambda solver, u, t, r: solver.applied.append((u, t, r)))
    monkeypatch.setattr(autotune, "current", lambda solver: dict(zip(("unroll", "threads", "resident_bytes"),
                                                                     solver.applied[-1])))
    monkeypatch.setattr(autotune, "measure", lambda solver, frame, restore, frames:
                        {"us_per_iteration": timings[solver.applied[-1]], "launch_ms": 1.0, "iterations": 9.0})


def test_picks_fastest_and_applies_it(monkeypatch, tmp_path):
    cands = [(4, 1024, 0), (2, 1024, 0), (4, 256, 0)]
    timings = {(4, 1024, 0): 75.0, (2, 1024, 0): 74.0, (4, 256, 0): 80.0}
    _patch(monkeypatch, tmp_path, timings)
    s = FakeSolver()
    best = autotune.autotune(s, None, None, candidates=cands, use_cache=False)
    assert (best["unroll"], best["threads"]) == (2, 1024)
    assert s.applied[-1] == (2, 1024, 0)
    assert s.applied[:3] == cands


def test_cache_round_trip_skips_measurement(monkeypatch, tmp_path):
    cands = [(4, 1024, 0), (4, 512, 0)]
    _patch(monkeypatch, tmp_path, {(4, 1024, 0): 70.0, (4, 512, 0): 72.0})
    first = autotune.autotune(FakeSolver(), None, None, candidates=cands)
    assert json.loads((tmp_path / "tune.json").read_text())["fake-gpu|P=8"]["threads"] == 1024
    monkeypatch.setattr(autotune, "measure", lambda *a: (_ for _ in ()).throw(AssertionError("measured again")))
    s = FakeSolver()
    again = autotune.autotune(s, None, None, candidates=cands)
    assert again == first and s.applied == [(4, 1024, 0)]


def test_default_candidates_cover_cta_sizes():
    threads = {t for _, t, _ in autotune.DEFAULT_CANDIDATES}
    assert threads == {256, 512, 1024}
    assert all(r == -2 for _, _, r in autotune.DEFAULT_CANDIDATES)  # automatic L2 residency
