"""latticeqmc_gb300 -- GB300-native DQMC sweep engine behind lqmc's API.

Drop-in for KieDani/LatticeQMC's ``lqmc`` package (lqmc/__init__.py:9-96): the model,
lattice, configuration and solver classes and the ``measure`` / ``measure_betas`` entry
points, with the sweep hot path running as hand-written sm_103a CUDA (liblqmc_gpu.so).
The reference's process pool (lqmc/multiprocessing.py) is replaced by independent chains
batched on the device.
"""
import os

import numpy as np

from .configuration import Configuration
from .engine import ChainSpec, Engine
from .hubbard import HubbardModel
from .lattice import Lattice
from .lqmc import LatticeQMC
from .managers import ParallelProcessManager, SerialProcessManager
from .scans import scan
from .tools import (check_params, compute_pole_gf_tau, decompose, fermi_fct, filling,
                    get_datapath, local_gf, local_moment, matsubara_frequencies, pole_gf_tau,
                    reconstruct)

__all__ = ["Configuration", "ChainSpec", "Engine", "HubbardModel", "Lattice", "LatticeQMC",
           "ParallelProcessManager", "SerialProcessManager", "measure", "measure_betas", "scan",
           "check_params", "compute_pole_gf_tau", "decompose", "fermi_fct", "filling",
           "get_datapath", "local_gf", "local_moment", "matsubara_frequencies", "pole_gf_tau",
           "reconstruct"]

_DEFAULT_CHAINS = 16


def _split_sweeps(sweeps, n):
    """Measurement sweeps per chain as ParallelProcessManager.set_jobs (multiprocessing.py:260-263)."""
    per = np.full(n, sweeps / n, dtype="int")
    per[0] += sweeps - np.sum(per)
    return per


def measure(model, beta, time_steps, warmup, sweeps, cores=None, det_mode=False, **engine_kw):
    """Warm up and measure G for `model` (lqmc/__init__.py:17-54).

    cores == 1 runs one chain through LatticeQMC exactly as the reference.  Otherwise
    `cores` (default 16) independent chains run batched on the GPU, each with `warmup`
    warm-up sweeps and an equal share of `sweeps`; the result is the sweep-weighted mean
    of their G.  Extra keywords (mode, rng, stab_every, seed, device) go to the engine.
    """
    if cores is not None and cores == 1:
        solver = LatticeQMC(model, beta, time_steps, warmup, sweeps, det_mode, **engine_kw)
        gf_up, gf_dn = solver.run()
        return gf_up, gf_dn
    n = cores if cores and cores > 0 else _DEFAULT_CHAINS
    check_params(model.u, model.t, beta / time_steps)
    mode = engine_kw.pop("mode", None) or ("dqmc" if det_mode else "compat")
    rng = engine_kw.pop("rng", "philox")
    seed = engine_kw.pop("seed", None)
    if seed is None:
        seed = int(np.random.randint(0, 2 ** 31))
    per = _split_sweeps(sweeps, n)
    kin = model.ham_kinetic()
    specs = [ChainSpec(kin, model.u, beta, time_steps, Configuration(model.n_sites, time_steps).config)
             for _ in range(n)]
    return _run_batch(specs, warmup, per, mode, rng, seed, engine_kw)[0]


def _run_batch(specs, warmup, per_chain_sweeps, mode, rng, seed, engine_kw):
    eng = Engine(specs, mode=mode, rng=rng, seed=seed, **engine_kw)
    try:
        if rng == "replay":
            raise ValueError("batched runs draw their uniforms on the device (rng='philox')")
        eng.sweep(warmup, measure=False)
        eng.reset_measurements()
        # every chain is measured for exactly its share: all chains sweep together, and a
        # chain whose share is used up keeps the sums it had then (the extra sweeps of
        # the longer shares still advance it, unmeasured in effect)
        per = np.asarray(per_chain_sweeps, dtype=np.int64)
        done, kept = 0, {}
        for share in np.unique(per):
            if share > done:
                eng.sweep(int(share - done), measure=True)
                done = int(share)
            for c in np.nonzero(per == share)[0]:
                if share < per.max():
                    kept[int(c)] = (eng.green_sum(int(c))[0], eng.observables_raw(int(c)))
        for c, (gsum, obs) in kept.items():
            eng.set_measurement_sums(c, gsum, obs)
        results = []
        for c in range(len(specs)):
            gsum, cnt = eng.green_sum(c)
            results.append((gsum, cnt))
        tot = sum(r[0] for r in results)
        cnt = sum(r[1] for r in results)
        mean = tot / max(cnt, 1)
        return (mean[0], mean[1]), results
    finally:
        eng.close()


def measure_betas(model, betas, time_steps, warmup=500, sweeps=5000, cores=-1, caching=True,
                  det_mode=False, **engine_kw):
    """G for every inverse temperature in `betas` (lqmc/__init__.py:57-96).

    One chain per beta, all betas batched into one GPU launch (the reference ran one
    process per beta, lqmc/multiprocessing.py:292-341).  With `caching`, finished betas are
    kept in ``tmp_gf_series.npz`` while running and resumed from it, and the file is
    removed at the end, as SerialProcessManager does (multiprocessing.py:312-341).
    Returns (gf_up, gf_dn), each (M, N, N).
    """
    betas = np.atleast_1d(np.asarray(betas, dtype=np.float64))
    tmp_file = "tmp_gf_series.npz"
    results = [None] * len(betas)
    if caching and os.path.isfile(tmp_file):
        data = np.load(tmp_file, allow_pickle=True)
        if len(data["data"]) == len(betas) and np.allclose(data["beta"], betas):
            results = list(data["data"])
    todo = [i for i, r in enumerate(results) if r is None]
    if todo:
        mode = engine_kw.pop("mode", None) or ("dqmc" if det_mode else "compat")
        rng = engine_kw.pop("rng", "philox")
        seed = engine_kw.pop("seed", None)
        if seed is None:
            seed = int(np.random.randint(0, 2 ** 31))
        kin = model.ham_kinetic()
        specs = [ChainSpec(kin, model.u, betas[i], time_steps,
                           Configuration(model.n_sites, time_steps).config) for i in todo]
        _, per = _run_batch(specs, warmup, np.full(len(specs), sweeps), mode, rng, seed, engine_kw)
        for j, i in enumerate(todo):
            gsum, cnt = per[j]
            results[i] = gsum / max(cnt, 1)
        if caching:
            np.savez(tmp_file, beta=betas, data=np.array(results, dtype=object), allow_pickle=True)
    gf_data = np.array([np.asarray(r, dtype=np.float64) for r in results])
    if caching and os.path.isfile(tmp_file):
        os.remove(tmp_file)
    gf_up, gf_dn = np.swapaxes(gf_data, 0, 1)
    return gf_up, gf_dn
