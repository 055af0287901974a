"""Multi-GPU host logic for the batched path: scene sharding and replica timing.

The single-mesh step does not shard (one mesh is one linear system), so
several GPUs run independent replicas.  Batched independent scenes shard by
scene with no collective in the data path: each rank builds a handle over its
own scenes and steps them alone.  The only exchanges are host-side: the
maximum of the ranks' timings and an optional gather of the results.

``partition_scenes`` splits the scenes into contiguous ranges whose weights
(for example the number of stored matrix blocks, which sets the PCG cost) are
balanced: the largest rank weight is the smallest possible for contiguous
ranges, found by binary search over the bottleneck.
"""

from __future__ import annotations

import numpy as np
import torch
import torch.distributed as dist


def partition_scenes(weights, world_size: int) -> list[range]:
    """Contiguous scene ranges, one per rank, minimising the largest summed weight.

    ``weights`` are non-negative per-scene costs.  Every scene belongs to
    exactly one range; ranges are in scene order and may be empty when there
    are more ranks than scenes.
    """
    w = np.asarray(weights, dtype=np.float64)
    if world_size < 1:
        raise ValueError("world_size must be at least 1")
    if np.any(w < 0) or not np.all(np.isfinite(w)):
        raise ValueError("scene weights must be finite and non-negative")
    n = len(w)
    if n == 0:
        return [range(0, 0) for _ in range(world_size)]

    def cuts_for(limit):
        cuts, acc = [0], 0.0
        for i, x in enumerate(w):
            if acc + x > limit and acc > 0:
                cuts.append(i)
                acc = 0.0
            acc += x
        cuts.append(n)
        return cuts

    lo, hi = float(w.max()), float(w.sum())
    for _ in range(100):
        if hi - lo <= 1e-9 * max(1.0, hi):
            break
        mid = 0.5 * (lo + hi)
        if len(cuts_for(mid)) - 1 <= world_size:
            hi = mid
        else:
            lo = mid
    cuts = cuts_for(hi)
    ranges = [range(cuts[k], cuts[k + 1]) for k in range(len(cuts) - 1)]
    ranges += [range(n, n) for _ in range(world_size - len(ranges))]
    return ranges


def local_offsets(scene_offsets, scenes: range):
    """Node range and rebased scene offsets of a contiguous scene range."""
    off = np.asarray(scene_offsets, dtype=np.int64)
    lo, hi = int(off[scenes.start]), int(off[scenes.stop])
    return lo, hi, off[scenes.start:scenes.stop + 1] - lo


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of a per-rank float over the default process group (identity without one)."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_scene_results(local: torch.Tensor, scene_offsets, ranges: list[range], dst: int = 0):
    """Reassemble per-rank node arrays (each rank's scene range, in order) on rank ``dst``.

    Returns the full ``[nodes, ...]`` tensor on ``dst`` and None elsewhere.  CPU
    tensors work with the gloo backend; device tensors with NCCL.
    """
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return local
    rank, world = dist.get_rank(), dist.get_world_size()
    off = np.asarray(scene_offsets, dtype=np.int64)
    sizes = [int(off[r.stop] - off[r.start]) for r in ranges]
    if local.shape[0] != sizes[rank]:
        raise ValueError("local result does not match this rank's scene range")
    trailing = tuple(local.shape[1:])
    parts = [torch.empty((sizes[k],) + trailing, dtype=local.dtype, device=local.device) for k in range(world)] \
        if rank == dst else None
    if rank == dst:
        parts[rank].copy_(local)
        for k in range(world):
            if k != rank and sizes[k] > 0:
                dist.recv(parts[k], src=k)
        return torch.cat(parts, dim=0)
    if sizes[rank] > 0:
        dist.send(local.contiguous(), dst=dst)
    return None
