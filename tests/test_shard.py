"""Voxel sharding (replicas, no data-path collective) on world_size-2 gloo ranks, CPU.

Each rank fits its own voxel range with the CPU oracle standing in for the
GPU fit (the sharding and merging logic is what is tested), the ranks'
results are gathered, and the merge must equal the unsharded fit (the same
selected pairs; values up to the rounding of other batch sizes).
"""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from fastfuncstuff_gb300.glm.arma import ARMA11Results
from fastfuncstuff_gb300.glm.shard import gather_results, shard_bounds
from oracle import reml as o
from tests.conftest import load_golden

FIELDS = ("betas", "tstats", "sigma2", "arma_params", "reml_likelihood")


def _fit(Y, d) -> ARMA11Results:
    ref = o.fit_glm_arma11(Y, d["X"], a_grid=d["a_grid"], b_grid=d["b_grid"], use_double=True)
    res = ARMA11Results()
    for f in FIELDS:
        setattr(res, f, torch.from_numpy(np.ascontiguousarray(getattr(ref, f))))
    return res


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        d = load_golden("single")
        V = d["Y"].shape[0]
        v0, v1 = shard_bounds(V, world, rank)
        merged = gather_results(_fit(d["Y"][v0:v1], d), V)
        if rank == 0:
            q.put({f: getattr(merged, f).numpy() for f in FIELDS})
    finally:
        dist.destroy_process_group()


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_bounds_cover_and_balance():
    for V in (0, 1, 7, 240, 200_001):
        for world in (1, 2, 3, 8):
            b = [shard_bounds(V, world, r) for r in range(world)]
            assert b[0][0] == 0 and b[-1][1] == V
            assert all(b[r][1] == b[r + 1][0] for r in range(world - 1))
            sizes = [v1 - v0 for v0, v1 in b]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(10, 2, 2)


def test_two_rank_gloo_merge_equals_unsharded_fit():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    d = load_golden("single")
    want = _fit(d["Y"], d)
    # the same voxels in other batch sizes: equal up to the BLAS blocking's rounding
    np.testing.assert_array_equal(got["arma_params"], want.arma_params.numpy())
    for f in FIELDS:
        np.testing.assert_allclose(got[f], getattr(want, f).numpy(), rtol=1e-10, atol=1e-12)
