"""Multi-process chain sharding and merge on CPU: world_size 2 over the gloo backend."""
import os
import socket

import numpy as np
import pytest

from latticeqmc_gb300.distributed import max_over_ranks, merge_sums, rank_seed, shard_chains


def test_shard_chains_covers_every_chain_once_balanced():
    for n, world in ((512, 8), (64, 3), (5, 4), (3, 5)):
        blocks = [shard_chains(n, r, world) for r in range(world)]
        flat = [i for b in blocks for i in b]
        assert flat == list(range(n))
        sizes = [len(b) for b in blocks]
        assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_chains(4, 2, 2)


def test_rank_seeds_distinct():
    seeds = {rank_seed(7, r) for r in range(64)}
    assert len(seeds) == 64
    assert rank_seed(7, 0) != rank_seed(8, 0)


def test_merge_single_process_is_sweep_weighted_mean():
    rng = np.random.default_rng(0)
    g = rng.random((3, 2, 4, 4))
    c = np.array([10, 20, 30])
    o = rng.random((3, 4))
    mean, omean, total = merge_sums(g, c, o)
    assert total == 60
    np.testing.assert_allclose(mean, g.sum(0) / 60)
    np.testing.assert_allclose(omean, o.sum(0) / 60)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n_chains, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # every chain's sums are a deterministic function of its global index, standing in
        # for what the GPU engine accumulates; uneven measurement counts per chain
        mine = shard_chains(n_chains, rank, world)
        g = np.stack([np.full((2, 3, 3), float(i + 1)) * (i + 2) for i in mine])
        cnt = np.array([i + 2 for i in mine])
        obs = np.stack([np.arange(4.0) * (i + 2) for i in mine])
        mean, omean, total = merge_sums(g, cnt, obs)
        tmax = max_over_ranks(10.0 + rank)
        np.savez(os.path.join(out_dir, f"r{rank}.npz"), mean=mean, omean=omean, total=total,
                 tmax=tmax)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_merge_to_the_single_process_answer(tmp_path):
    import torch.multiprocessing as tmp
    n_chains, world = 7, 2
    port = _free_port()
    tmp.spawn(_worker, args=(world, port, n_chains, str(tmp_path)), nprocs=world, join=True)
    # single-process answer
    idx = np.arange(n_chains)
    g = np.stack([np.full((2, 3, 3), float(i + 1)) * (i + 2) for i in idx])
    cnt = idx + 2
    ref = g.sum(0) / cnt.sum()
    for r in range(world):
        f = np.load(tmp_path / f"r{r}.npz")
        np.testing.assert_allclose(f["mean"], ref)
        np.testing.assert_allclose(f["omean"], np.arange(4.0) * cnt.sum() / cnt.sum())
        assert int(f["total"]) == cnt.sum()
        assert float(f["tmax"]) == 11.0


def _worker_too_few(rank, world, port, out_dir):
    import torch.distributed as dist
    from latticeqmc_gb300.distributed import run_local_chains
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        raised = ""
        try:
            # one chain for two ranks: every rank must refuse before building an engine or
            # entering a collective
            run_local_chains([object()], warmup=1, sweeps=1, rank=rank, world=world)
        except ValueError as e:
            raised = str(e)
        dist.barrier()
        np.savez(os.path.join(out_dir, f"few{rank}.npz"), raised=raised)
    finally:
        dist.destroy_process_group()


def test_fewer_chains_than_ranks_raises_on_every_rank(tmp_path):
    import torch.multiprocessing as tmp
    world = 2
    tmp.spawn(_worker_too_few, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    for r in range(world):
        msg = str(np.load(tmp_path / f"few{r}.npz")["raised"])
        assert "cannot be shared by 2 ranks" in msg
