"""The reference's process managers (lqmc/multiprocessing.py:55-341) with the same names and
calls, backed by chains batched on the GPU instead of a pool of CPU processes.

Callers of the reference use them as lqmc/__init__.py:17-96 does:

    manager = ParallelProcessManager(model, beta, time_steps, warmup, det_mode, procs=cores)
    manager.set_jobs(sweeps)
    manager.run()
    gf = manager.get_result()          # (2, N, N)
    manager.terminate()

    manager = SerialProcessManager(model, time_steps, warmup, sweeps, det_mode, cores, caching)
    manager.set_jobs(betas)
    manager.run(sleep=1.0)
    gf_data = manager.get_result()     # (M, 2, N, N), one entry per beta
    manager.terminate()

``procs`` becomes the number of chains (ParallelProcessManager; the reference's one chain
per process) and is not used by SerialProcessManager, which batches every beta in one launch.
Keyword arguments the GPU engine adds (mode, precision, rng, seed, ...) are passed through.
The result of ParallelProcessManager is the sweep-weighted mean over chains; the
reference's unweighted mean over processes (lqmc/multiprocessing.py:265-267) differs from it
only when the sweeps do not split evenly.
"""
import os

import numpy as np


class _Manager:
    def __init__(self, procs=None, **default_kwargs):
        self.max_procs = procs
        self.default_kwargs = dict(default_kwargs)
        self.var_kwargs = {}
        self.result = None

    @property
    def model(self):
        return self.default_kwargs["model"]

    @property
    def all_done(self):
        return self.result is not None

    def join(self):
        pass

    def terminate(self):
        pass


class ParallelProcessManager(_Manager):
    """G of one model at one beta from ``procs`` independent chains."""

    def __init__(self, model, beta, time_steps, warmup=300, det_mode=False, procs=None,
                 **engine_kw):
        super().__init__(procs, model=model, beta=beta, time_steps=time_steps, warmup=warmup,
                         det_mode=det_mode)
        self.engine_kw = engine_kw

    def set_jobs(self, sweeps):
        """Total measurement sweeps, split over the chains as lqmc/multiprocessing.py:260-263."""
        self.var_kwargs = {"sweeps": int(sweeps)}
        self.result = None

    def run(self, sleep=0.5):
        from . import measure
        k = self.default_kwargs
        gf_up, gf_dn = measure(k["model"], k["beta"], k["time_steps"], k["warmup"],
                               self.var_kwargs["sweeps"], cores=self.max_procs,
                               det_mode=k["det_mode"], **self.engine_kw)
        self.result = np.array([gf_up, gf_dn])

    def get_result(self):
        return self.result


class SerialProcessManager(_Manager):
    """G of one model at every beta of a list, one chain per beta."""

    def __init__(self, model, time_steps, warmup=300, sweeps=2000, det_mode=False, procs=None,
                 caching=True, **engine_kw):
        super().__init__(procs, model=model, time_steps=time_steps, warmup=warmup,
                         sweeps=sweeps, det_mode=det_mode)
        self.caching = caching
        self.engine_kw = engine_kw
        self._tmp_file = "tmp_gf_series.npz"     # the cache measure_betas keeps while running

    def set_jobs(self, betas):
        self.var_kwargs = {"beta": np.atleast_1d(np.asarray(betas, dtype=np.float64))}
        self.result = None

    def run(self, sleep=1.0):
        from . import measure_betas
        k = self.default_kwargs
        gf_up, gf_dn = measure_betas(k["model"], self.var_kwargs["beta"], k["time_steps"],
                                     warmup=k["warmup"], sweeps=k["sweeps"],
                                     caching=self.caching, det_mode=k["det_mode"],
                                     **self.engine_kw)
        self.result = np.swapaxes(np.array([gf_up, gf_dn]), 0, 1)

    def delete_cache(self):
        """Remove ``tmp_gf_series.npz`` from the working directory: the resume cache that
        measure_betas writes while it runs with caching=True (the reference's manager keeps its
        cache under the same name, lqmc/multiprocessing.py:313-333, so one left by an
        interrupted reference run in the same directory is removed too)."""
        if os.path.isfile(self._tmp_file):
            os.remove(self._tmp_file)

    def get_result(self):
        return self.result
