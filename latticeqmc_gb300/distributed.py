"""Independent chains over several GPUs (one process per GPU).

The reference's pool runs one chain per process and averages the per-process mean G
(lqmc/multiprocessing.py:252-267); its mean is unweighted, which is slightly wrong when the
sweep split is uneven (:260-263).  Here each rank runs its own block of chains on its own
GPU with its own Philox key, there is no exchange while sweeping, and the only collective is
one sum of the measurement accumulators at the end: the result is the sweep-weighted mean
over all chains of all ranks.
"""
import numpy as np


def shard_chains(n_chains, rank, world):
    """Contiguous, balanced block of chain indices owned by `rank` (sizes differ by <= 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    base, extra = divmod(n_chains, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return list(range(lo, hi))


def rank_seed(seed, rank):
    """Philox key word of a rank: distinct per rank for the same base seed."""
    x = (int(seed) * 0x9E3779B97F4A7C15 + (int(rank) + 1) * 0xBF58476D1CE4E5B9) & ((1 << 64) - 1)
    x ^= x >> 31
    return x


def merge_sums(green_sums, counts, obs_sums=None, group=None):
    """Sweep-weighted mean over all ranks.

    green_sums : (n_local, 2, N, N) sums of G of this rank's chains (same N on every rank)
    counts     : (n_local,) measurements per chain
    obs_sums   : optional (n_local, M) observable sums
    Returns (mean G (2, N, N), mean observables (M,) or None, total measurements).
    Uses torch.distributed when it is initialised (any backend), else this process alone.
    """
    import torch
    import torch.distributed as dist
    g = np.asarray(green_sums, dtype=np.float64).sum(axis=0)
    c = float(np.sum(counts))
    o = None if obs_sums is None else np.asarray(obs_sums, dtype=np.float64).sum(axis=0)
    if dist.is_available() and dist.is_initialized():
        dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
        parts = [g.ravel(), np.array([c])] + ([] if o is None else [o.ravel()])
        flat = torch.from_numpy(np.concatenate(parts)).to(dev)
        dist.all_reduce(flat, op=dist.ReduceOp.SUM, group=group)
        flat = flat.cpu().numpy()
        g = flat[:g.size].reshape(g.shape)
        c = float(flat[g.size])
        if o is not None:
            o = flat[g.size + 1:].reshape(o.shape)
    if c <= 0:
        raise ValueError("no measurements to merge")
    return g / c, (None if o is None else o / c), int(round(c))


def max_over_ranks(value, group=None):
    """The largest `value` over all ranks (the step time a multi-GPU run reports)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def run_local_chains(specs, warmup, sweeps, rank, world, seed=0, **engine_kw):
    """Sweep this rank's block of `specs` on its GPU and merge with the other ranks.

    Returns (mean G, mean observables vector, total measurements) over every chain of every
    rank.  All ranks must pass the same `specs` list."""
    from .engine import Engine
    # every rank checks the same condition on the same `specs` before any collective, so
    # too few chains raise the same error everywhere instead of leaving ranks waiting in
    # the final all_reduce
    if len(specs) < world:
        raise ValueError(f"{len(specs)} chains cannot be shared by {world} ranks: every rank "
                         "needs at least one chain")
    mine = [specs[i] for i in shard_chains(len(specs), rank, world)]
    eng = Engine(mine, rng="philox", seed=rank_seed(seed, rank), **engine_kw)
    try:
        eng.sweep(warmup)
        eng.reset_measurements()
        eng.sweep(sweeps, measure=True)
        gs, cs, os_ = [], [], []
        for c in range(len(mine)):
            g, n = eng.green_sum(c)
            gs.append(g)
            cs.append(n)
            os_.append(eng.observables_raw(c)[1:5])
    finally:
        eng.close()
    return merge_sums(np.array(gs), np.array(cs), np.array(os_))
