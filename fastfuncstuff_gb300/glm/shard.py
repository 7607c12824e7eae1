"""Voxel sharding across processes (one GPU each): replicas, no data-path collective.

The REML fit of one voxel does not depend on any other voxel, so N processes
fit N disjoint voxel ranges with no exchange during the fit. ``shard_bounds``
gives each rank its contiguous range; ``gather_results`` assembles the ranks'
per-voxel result arrays on every rank afterwards (one all-gather per field over
the caller's process group: gloo on the host, or NCCL with device tensors).
"""

from __future__ import annotations

import torch

from .arma import VOXEL_SCATTER_ATTRS, ARMA11Results


def shard_bounds(n_voxels: int, world: int, rank: int) -> tuple[int, int]:
    """[v0, v1) of rank ``rank`` of ``world``: contiguous, sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    base, extra = divmod(int(n_voxels), world)
    v0 = rank * base + min(rank, extra)
    return v0, v0 + base + (1 if rank < extra else 0)


def gather_results(local: ARMA11Results, n_voxels: int, group=None) -> ARMA11Results:
    """Every rank's per-voxel fields concatenated in rank order (the fit of
    voxels [0, n_voxels)); the other fields are taken from the local result.
    Ranks must hold the same set of fields. Collective over ``group``."""
    import copy

    import torch.distributed as dist

    world = dist.get_world_size(group)
    out = copy.copy(local)
    for attr in VOXEL_SCATTER_ATTRS:
        t = getattr(local, attr, None)
        if t is None:
            continue
        sizes = [shard_bounds(n_voxels, world, r) for r in range(world)]
        n_max = max(v1 - v0 for v0, v1 in sizes)
        pad = torch.zeros((n_max,) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)
        pad[: t.shape[0]] = t
        parts = [torch.empty_like(pad) for _ in range(world)]
        dist.all_gather(parts, pad, group=group)
        setattr(out, attr, torch.cat([p[: v1 - v0] for p, (v0, v1) in zip(parts, sizes)]))
    return out
