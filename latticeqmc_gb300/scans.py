"""Batched (U, beta) scans with per-chain checkpoint / resume.

The reference runs one process per point of a scan (`SerialProcessManager`,
lqmc/multiprocessing.py:292-341, driven by lqmc/__init__.py:57-96 and comp.py:19-47) and can
only cache finished points (`tmp_gf_series.npz`).  Here every chain of every point runs in one
engine (one launch per sweep for all of them), and the whole batch is checkpointed every
`checkpoint_every` sweeps: fields, the Philox sweep counters and the measurement sums, so an
interrupted scan resumes exactly where it stopped and ends with the same numbers as an
uninterrupted one.
"""
import os

import numpy as np

from .engine import ChainSpec, Engine


def scan(kinetic, points, time_steps, warmup, sweeps, chains_per_point=1, seed=0,
         checkpoint=None, checkpoint_every=100, stop_after=None, **engine_kw):
    """Measure every (u, beta) point of `points` on the lattice with hopping matrix `kinetic`.

    time_steps  L (slices per point; dtau = beta / L)
    warmup, sweeps  per chain
    chains_per_point  independent chains per point (fields from a per-point seeded stream)
    checkpoint  .npz path: resumed from when it exists, rewritten every `checkpoint_every`
                sweeps and removed when the scan completes
    stop_after  stop (after writing the checkpoint) once this call has run that many sweeps;
                for jobs with a wall-clock limit
    Remaining keywords go to `Engine` (mode defaults to 'dqmc', precision, stab_every, ...).

    Returns a dict of arrays: u, beta (P,), green (P, 2, N, N) mean G, count (P,)
    measurements, and per-point means of the Wick observables (kinetic_energy,
    potential_energy, double_occupancy, density); or None when stopped early.
    """
    pts = [(float(u), float(b)) for u, b in points]
    if not pts:
        raise ValueError("no scan points")
    kin = np.asarray(kinetic, dtype=np.float64)
    n = kin.shape[0]
    specs, owner = [], []
    for p, (u, beta) in enumerate(pts):
        rng = np.random.default_rng([seed, p])
        for _ in range(chains_per_point):
            field = (2 * rng.integers(0, 2, (n, time_steps)) - 1).astype(np.int8)
            specs.append(ChainSpec(kin, u, beta, time_steps, field))
            owner.append(p)
    engine_kw.setdefault("mode", "dqmc")
    eng = Engine(specs, rng="philox", seed=seed, **engine_kw)
    try:
        if checkpoint and os.path.isfile(checkpoint):
            eng.restore(checkpoint)
        done = int(eng.diagnostics(0)["sweeps"])
        total = warmup + sweeps
        ran = 0
        while done < total:
            if stop_after is not None and ran >= stop_after:
                return None
            limit = total - done
            if stop_after is not None:
                limit = min(limit, stop_after - ran)
            if checkpoint:
                limit = min(limit, checkpoint_every)
            measuring = done >= warmup
            if not measuring:
                limit = min(limit, warmup - done)
            if measuring and done == warmup:
                eng.reset_measurements()
            eng.sweep(limit, measure=measuring)
            done += limit
            ran += limit
            if checkpoint and done < total:
                eng.checkpoint(checkpoint)
        out = {"u": np.array([p[0] for p in pts]), "beta": np.array([p[1] for p in pts]),
               "green": np.zeros((len(pts), 2, n, n)), "count": np.zeros(len(pts), dtype=np.int64)}
        obs_keys = ("kinetic_energy", "potential_energy", "double_occupancy", "density")
        sums = {k: np.zeros(len(pts)) for k in obs_keys}
        for c, p in enumerate(owner):
            g, cnt = eng.green_sum(c)
            out["green"][p] += g
            out["count"][p] += cnt
            raw = eng.observables_raw(c)
            for j, k in enumerate(obs_keys):
                sums[k][p] += raw[1 + j]
        for p in range(len(pts)):
            out["green"][p] /= max(int(out["count"][p]), 1)
        for k in obs_keys:
            out[k] = sums[k] / np.maximum(out["count"], 1)
        if checkpoint and os.path.isfile(checkpoint):
            os.remove(checkpoint)
        return out
    finally:
        eng.close()
