"""PCG launch tuning on the GPU (``-m gpu``): every launch variant solves the same system.

The variants (SpMV unroll, CTA size, resident row-state layout, row split by
calibrated CTA speed, the single-reduction CG recurrence) change only the
summation order of the grid reductions, where row state lives or the rounding of
mathematically equal recurrences, so a substep agrees with the default
configuration to float32 round-off (relative 1e-5 on the velocity increment at a
tight tolerance), and repeated substeps of one configuration are bit-identical.
"""

import ctypes

import numpy as np
import pytest
import torch
from gpu_helpers import rel_l2, scene_pair, to_np

from newton_solver_fem_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _cuda(cuda_device):
    yield


def setting(solver, key):
    v = ctypes.c_int64()
    _lib.check(_lib.load().fem_get_tuning(solver._handle, key, ctypes.byref(v)))
    return v.value


def substep(model, solver, sc):
    solver.reset()
    s0, s1 = model.state(), model.state()
    solver.refresh_tangent(s0.particle_q)
    solver.step(s0, s1, None, None, sc.dt)
    torch.cuda.synchronize()
    return to_np(solver.velocity_increment), to_np(s1.particle_q)


VARIANTS = [
    {_lib.FEM_TUNE_SPMV_UNROLL: 1},
    {_lib.FEM_TUNE_SPMV_UNROLL: 2},
    {_lib.FEM_TUNE_CTA_THREADS: 1024},
    {_lib.FEM_TUNE_CTA_THREADS: 512, _lib.FEM_TUNE_GRID_CAP: 7},
    {_lib.FEM_TUNE_RESIDENT_LAYOUT: 0},
    {_lib.FEM_TUNE_RESIDENT_LAYOUT: 2},
    {_lib.FEM_TUNE_BALANCE: 1},
    {_lib.FEM_TUNE_RESIDENT_LAYOUT: 2, _lib.FEM_TUNE_BALANCE: 1},
    {_lib.FEM_TUNE_SPLIT_HEADROOM: 10, _lib.FEM_TUNE_BALANCE: 1},
    {_lib.FEM_TUNE_TAIL_PREFETCH: 0},
    {_lib.FEM_TUNE_TAIL_PREFETCH: 100},
    {_lib.FEM_TUNE_COMPACT_COLUMNS: 0},
    {_lib.FEM_TUNE_COMPACT_COLUMNS: 1},
    {_lib.FEM_TUNE_COMPACT_COLUMNS: 2},
    {_lib.FEM_TUNE_COMPACT_COLUMNS: 2, _lib.FEM_TUNE_SPMV_UNROLL: 1},
    {_lib.FEM_TUNE_L2_RESIDENT_BYTES: 0},
    {_lib.FEM_TUNE_L2_RESIDENT_BYTES: 1 << 20, _lib.FEM_TUNE_COMPACT_COLUMNS: 2},
    {_lib.FEM_TUNE_CG_VARIANT: 1},
    {_lib.FEM_TUNE_CG_VARIANT: 1, _lib.FEM_TUNE_RESIDENT_LAYOUT: 0},
    {_lib.FEM_TUNE_CG_VARIANT: 1, _lib.FEM_TUNE_RESIDENT_LAYOUT: 2},
    {_lib.FEM_TUNE_CG_VARIANT: 1, _lib.FEM_TUNE_COMPACT_COLUMNS: 1, _lib.FEM_TUNE_SPMV_UNROLL: 2},
    {_lib.FEM_TUNE_CG_VARIANT: 1, _lib.FEM_TUNE_BALANCE: 1},
]


@pytest.mark.parametrize("variant", VARIANTS, ids=lambda v: "-".join(f"{k}={x}" for k, x in v.items()))
def test_launch_variants_solve_the_same_system(variant):
    sc = scenes.hex_block_64(n=24)
    model, solver, _ = scene_pair(sc, linear_solver_tolerance=1e-6, linear_solver_maxiter=400, with_oracle=False)
    dv_ref, q_ref = substep(model, solver, sc)
    lib = _lib.load()
    for key, value in variant.items():
        _lib.check(lib.fem_set_tuning(solver._handle, key, value))
    for key, value in variant.items():
        assert setting(solver, key) == value
    dv, q = substep(model, solver, sc)
    dv2, q2 = substep(model, solver, sc)
    np.testing.assert_array_equal(dv, dv2)  # deterministic within a configuration
    np.testing.assert_array_equal(q, q2)
    assert rel_l2(dv, dv_ref) < 1e-5
    assert np.isfinite(dv).all()


def test_calibrated_split_survives_topology_refresh_and_rejects_bad_values():
    sc = scenes.tet_jittered_48(n=10)
    model, solver, _ = scene_pair(sc, with_oracle=False)
    lib = _lib.load()
    _lib.check(lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_BALANCE, 1))
    for key, bad in ((_lib.FEM_TUNE_BALANCE, 2), (_lib.FEM_TUNE_RESIDENT_LAYOUT, 3),
                     (_lib.FEM_TUNE_SPLIT_HEADROOM, -1), (_lib.FEM_TUNE_SPLIT_HEADROOM, 51),
                     (_lib.FEM_TUNE_TAIL_PREFETCH, 101)):
        assert lib.fem_set_tuning(solver._handle, key, bad) == _lib.FEM_ERR_BAD_ARG
    solver.refresh_topology(model.particle_q)
    assert setting(solver, _lib.FEM_TUNE_BALANCE) == 1
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, sc.dt)
    assert torch.isfinite(s1.particle_q).all()


def test_automatic_residency_and_column_mode():
    """A matrix that fits in 60% of L2 is kept there whole and read with per-row offsets; one that
    streams (no resident bytes) reads the offsets its slices share once per slice."""
    sc = scenes.hex_block_64(n=12)
    model, solver, _ = scene_pair(sc, with_oracle=False)
    lib = _lib.load()
    nslices = -(-model.particle_count // 32)
    assert setting(solver, _lib.FEM_TUNE_L2_RESIDENT_BYTES) == -2
    assert setting(solver, _lib.FEM_TUNE_RESIDENT_SLICES) == nslices
    assert setting(solver, _lib.FEM_TUNE_COMPACT_COLUMNS) == 1
    _lib.check(lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_L2_RESIDENT_BYTES, 0))
    assert setting(solver, _lib.FEM_TUNE_RESIDENT_SLICES) == 0
    assert setting(solver, _lib.FEM_TUNE_COMPACT_COLUMNS) == 2
    assert setting(solver, _lib.FEM_TUNE_UNIFORM_COLUMN_BLOCKS) > 0
    for key, bad in ((_lib.FEM_TUNE_L2_RESIDENT_BYTES, -3), (_lib.FEM_TUNE_COMPACT_COLUMNS, -2)):
        assert lib.fem_set_tuning(solver._handle, key, bad) == _lib.FEM_ERR_BAD_ARG


def test_column_modes_are_bit_identical_and_report_shared_slots():
    """Column modes only change where a block's column comes from, so substeps agree bit for bit."""
    sc = scenes.hex_block_64(n=12)
    model, solver, _ = scene_pair(sc, with_oracle=False)
    lib = _lib.load()
    _lib.check(lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_COMPACT_COLUMNS, 2))
    assert setting(solver, _lib.FEM_TUNE_COMPACT_COLUMNS) == 2
    shared = setting(solver, _lib.FEM_TUNE_UNIFORM_COLUMN_BLOCKS)
    assert 0 < shared < solver.matrix_info()["nnzb"]
    ref = substep(model, solver, sc)
    for mode in (1, 0):
        _lib.check(lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_COMPACT_COLUMNS, mode))
        assert setting(solver, _lib.FEM_TUNE_UNIFORM_COLUMN_BLOCKS) == 0
        got = substep(model, solver, sc)
        np.testing.assert_array_equal(got[0], ref[0])
        np.testing.assert_array_equal(got[1], ref[1])
    assert lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_COMPACT_COLUMNS, 3) == _lib.FEM_ERR_BAD_ARG


def test_calibrated_split_of_a_spread_batch():
    """A 24-scene batch (slices dealt to CTAs in interleaved runs) re-split by calibrated CTA speed
    solves the same system, deterministically."""
    sc = scenes.batched_scenes(count=24, seed=5, dims=(3, 10))
    model, solver, _ = scene_pair(sc, linear_solver_tolerance=1e-6, linear_solver_maxiter=200, with_oracle=False)
    dv_ref, _ = substep(model, solver, sc)
    lib = _lib.load()
    _lib.check(lib.fem_set_tuning(solver._handle, _lib.FEM_TUNE_BALANCE, 1))
    dv, _ = substep(model, solver, sc)
    dv2, _ = substep(model, solver, sc)
    np.testing.assert_array_equal(dv, dv2)
    assert rel_l2(dv, dv_ref) < 1e-5


def test_handles_needing_different_pcg_shared_memory_launch_in_any_order():
    """Two systems of 32 and 24 slices each run as one CTA (a warp per slice), whose PCG launches need
    about 79 KB and 60 KB of dynamic shared memory, above the default 48 KB.  That limit belongs to the
    kernel, not the handle; configuring the smaller system after the larger must leave the larger one's
    cooperative launch (eager and graph-captured) valid, and every step must match a fresh handle."""
    from gpu_helpers import make_pair

    def pair(cells):
        x, hexes, mats, mass = scenes.hex_block(*cells, 0.05, (0.0, 0.0, 0.0), 1e5, 0.3, 1000.0)
        return make_pair(x, mass, hexes=hexes, hex_materials=mats, gravity=(0.0, 0.0, -9.81), with_oracle=False,
                         linear_solver_maxiter=40, linear_solver_tolerance=1e-6)

    big_model, big, _ = pair((9, 9, 9))      # 1,000 nodes: 32 slices
    small_model, small, _ = pair((7, 7, 11))  # 768 nodes: 24 slices
    assert setting(big, _lib.FEM_TUNE_GRID) == 1 and setting(big, _lib.FEM_TUNE_CTA_THREADS) == 1024
    assert setting(small, _lib.FEM_TUNE_GRID) == 1 and setting(small, _lib.FEM_TUNE_CTA_THREADS) == 768

    def run(model, solver, steps=3):
        s0, s1 = model.state(), model.state()
        solver.reset()
        solver.refresh_tangent(s0.particle_q)
        for _ in range(steps):
            solver.step(s0, s1, None, None, 1.0 / 600.0)
            s0, s1 = s1, s0
        torch.cuda.synchronize()
        return to_np(s0.particle_q)

    q_big, q_small = run(big_model, big), run(small_model, small)
    again_model, again, _ = pair((9, 9, 9))
    assert np.array_equal(run(again_model, again), q_big)
    assert np.array_equal(run(big_model, big), q_big)  # after the small handle was configured
    assert np.array_equal(run(small_model, small), q_small)

    s0, s1 = big_model.state(), big_model.state()
    big.reset()
    graph = torch.cuda.CUDAGraph()
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        big.refresh_tangent(s0.particle_q)
        big.step(s0, s1, None, None, 1.0 / 600.0)  # allocations outside capture
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=stream):
            big.step(s0, s1, None, None, 1.0 / 600.0)
    pair((7, 7, 11))  # a third handle configured between capture and replay
    graph.replay()
    torch.cuda.synchronize()
    assert np.isfinite(to_np(s1.particle_q)).all()
