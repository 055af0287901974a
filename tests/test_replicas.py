"""Multi-process host logic on CPU: scene partitioning, max-over-ranks timing and the
result gather, with world_size-2 gloo process groups (no GPU)."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from newton_solver_fem_gb300 import replicas, scenes


def test_partition_covers_every_scene_once_and_balances():
    rng = np.random.default_rng(3)
    w = rng.integers(1, 1000, size=257)
    for world in (1, 2, 3, 8, 300):
        ranges = replicas.partition_scenes(w, world)
        assert len(ranges) == world
        flat = [i for r in ranges for i in r]
        assert flat == list(range(len(w)))
        loads = [w[list(r)].sum() if len(r) else 0 for r in ranges]
        # contiguous lower bound: no split can beat the mean or the heaviest scene
        assert max(loads) <= max(w.sum() / world, w.max()) + w.max()


def test_partition_is_optimal_on_small_cases():
    w = np.array([5, 1, 1, 1, 5, 1, 1, 1])
    ranges = replicas.partition_scenes(w, 2)
    assert [w[list(r)].sum() for r in ranges] == [8, 8]
    assert replicas.partition_scenes([], 3) == [range(0, 0)] * 3
    with pytest.raises(ValueError):
        replicas.partition_scenes([1, -1], 2)


def test_local_offsets_rebase_the_batched_scenes():
    sc = scenes.batched_scenes(count=6, seed=11, dims=(2, 5))
    counts = np.diff(sc.scene_offsets)
    ranges = replicas.partition_scenes(counts, 2)
    nodes = 0
    for r in ranges:
        lo, hi, local = replicas.local_offsets(sc.scene_offsets, r)
        assert local[0] == 0 and local[-1] == hi - lo
        nodes += hi - lo
    assert nodes == sc.scene_offsets[-1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, offsets, out_q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ranges = replicas.partition_scenes(np.diff(offsets), world)
        lo, hi, _ = replicas.local_offsets(offsets, ranges[rank])
        # each rank "steps" its scenes: node i ends at value 10 i (independent of the split)
        local = torch.arange(lo, hi, dtype=torch.float32).reshape(-1, 1).repeat(1, 3) * 10.0
        full = replicas.gather_scene_results(local, offsets, ranges)
        ms = replicas.max_over_ranks(1.5 + rank)
        if rank == 0:
            out_q.put((full.numpy().tolist(), ms))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_scenes_and_take_the_slowest_time():
    offsets = np.array([0, 4, 9, 10, 17, 20], dtype=np.int64)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, offsets, q)) for r in range(2)]
    for p in procs:
        p.start()
    full, ms = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    expect = (np.arange(20, dtype=np.float32).reshape(-1, 1).repeat(3, axis=1) * 10.0).tolist()
    assert full == expect
    assert ms == 2.5
