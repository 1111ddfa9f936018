"""The replica (multi-rank) host logic on CPU with the gloo backend, world
size 2: chain sharding, max over ranks, and the global min-ESS from the
ranks' traces equals the ESS of the concatenated trace on one process."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _ar1_trace(seed, K=200, C=6, d=3, phi=0.8):
    rng = np.random.default_rng(seed)
    x = np.zeros((K, C, d))
    for k in range(1, K):
        x[k] = phi * x[k - 1] + rng.standard_normal((C, d))
    return x


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    from geomjax_gb300 import distributed as D

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        trace = torch.as_tensor(_ar1_trace(100 + rank, C=5 + rank))  # ragged chain counts
        out[f"ess{rank}"] = D.global_min_ess(trace, chain_axis=1, sample_axis=0)
        out[f"max{rank}"] = D.max_over_ranks(1.5 + rank)
        full = D.gather_chains(trace, chain_axis=1)
        out[f"shape{rank}"] = tuple(full.shape)
    finally:
        dist.destroy_process_group()


def test_shard_covers_every_unit_once():
    from geomjax_gb300.distributed import shard

    for total in (0, 1, 7, 4096, 4097):
        for world in (1, 2, 3, 8):
            parts = [shard(total, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == total
            assert all(parts[r][1] == parts[r + 1][0] for r in range(world - 1))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1


def test_two_rank_gloo_global_ess_and_max():
    import torch.multiprocessing as mp

    from geomjax_gb300.diagnostics import effective_sample_size

    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        res = dict(out)
    full = np.concatenate([_ar1_trace(100, C=5), _ar1_trace(101, C=6)], axis=1)
    ref = float(torch.min(effective_sample_size(torch.as_tensor(full), chain_axis=1,
                                                sample_axis=0)))
    assert res["shape0"] == res["shape1"] == (200, 11, 3)
    assert abs(res["ess0"] - ref) < 1e-9 * ref and abs(res["ess1"] - ref) < 1e-9 * ref
    assert res["max0"] == res["max1"] == 2.5
