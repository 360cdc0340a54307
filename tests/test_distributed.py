"""The multi-GPU path on CPU: cost-balanced member shards and the all-reduced
ensemble coherence, checked with two gloo ranks against the single-process result."""

import os
import socket

import numpy as np
import torch.multiprocessing as mp

from pyofsschanged_gb300.ensemble import (coherence_g12, coherence_g12_distributed, expected_attempts,
                                          shard, sc_ensemble)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shards_partition_and_balance():
    members, _, _ = sc_ensemble(256)
    cost = [m.n * np.log2(m.n) * expected_attempts(m) for m in members]
    for world in (1, 2, 4, 8):
        parts = [shard(members, r, world) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(256))
        loads = [sum(cost[i] for i in p) for p in parts]
        assert max(loads) <= 1.1 * sum(loads) / world + max(cost)


def _rank(rank, world, port, spectra, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = spectra[rank::world]
    g = coherence_g12_distributed(mine)
    out[rank] = g
    dist.destroy_process_group()


def test_coherence_allreduce_matches_single_process():
    rng = np.random.default_rng(5)
    spectra = rng.standard_normal((9, 64)) + 1j * rng.standard_normal((9, 64))
    spectra += 3.0  # a coherent part
    ref = coherence_g12(spectra)
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank, args=(world, port, spectra, out), nprocs=world, join=True,
                           start_method="spawn")
        for r in range(world):
            np.testing.assert_allclose(out[r], ref, rtol=1e-12, atol=1e-15)


def _rank_sharded(rank, world, port, spectra, out):
    import torch.distributed as dist
    from pyofsschanged_gb300.ensemble import coherence_g12_distributed
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = spectra[rank:rank + 1]  # ranks beyond the member count get an empty shard
    out[rank] = coherence_g12_distributed(mine, n_bins=spectra.shape[1])
    dist.destroy_process_group()


def test_coherence_allreduce_with_empty_shards():
    """More ranks than members: the ranks without members contribute zero sums and
    every rank still gets the single-process |g12|."""
    rng = np.random.default_rng(7)
    spectra = rng.standard_normal((2, 32)) + 1j * rng.standard_normal((2, 32)) + 2.0
    ref = coherence_g12(spectra)
    world, port = 3, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank_sharded, args=(world, port, spectra, out), nprocs=world, join=True,
                           start_method="spawn")
        for r in range(world):
            np.testing.assert_allclose(out[r], ref, rtol=1e-12, atol=1e-15)
