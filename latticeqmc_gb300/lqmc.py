"""GPU-backed drop-in for ``lqmc.LatticeQMC`` (lqmc/lqmc.py:14-408).

Same constructor, attributes and loop methods as the reference solver; the sweep itself
(``_update_step``) runs on the GPU through liblqmc_gpu.so.  Extra keyword arguments choose
the engine:

mode        'compat' (default): the reference's fast-sweep arithmetic, defects included;
            fed the reference's field and uniform stream its accept/reject decisions are
            the reference's.  'dqmc': textbook, QR-stabilised DQMC.
rng         'replay' (default): one ``np.random.rand()`` per site from numpy's global
            generator, in sweep order, exactly as lqmc.py:317 draws them.  'philox': on device.
stab_every  slices between from-scratch refreshes of G (dqmc); default: the largest with
            stab_every * dtau <= 0.5.
precision   'fp64' (default); 'fp64e' (float64 G, every dense product a float64-accurate
            GEMM emulated on the tensor cores; dqmc mode); 'mixed' (float32, dqmc mode).
delay       delayed-update depth of the tiled kernel (0: automatic).
engine      'auto', 'smem' or 'tiled' (see Engine).
fp64e_native  product categories the fp64e engine keeps in native float64 (see Engine).
measure_tau also accumulate the unequal-time G(tau_l, 0) on every measured sweep (dqmc mode;
            read with green_tau()).

``det_mode=True`` runs the exact-ratio chain (mode 'dqmc'): its ratios equal the reference's
determinant ratios (lqmc.py:244-248) to rounding.
The reference's determinant mode itself (every ratio from det M of the flipped field,
lqmc.py:236-299) runs on the device through ``warmup_loop_det``, ``measure_loop_det`` and
``_update_step_det`` (engine mode 'det'; small lattices).
"""
import logging
import time

import numpy as np

from .configuration import Configuration
from .engine import ChainSpec, Engine, hs_coupling

DEBUG = logging.DEBUG
_log = logging.getLogger("latticeqmc_gb300")

# largest uniform block uploaded at once in replay mode (doubles)
_REPLAY_BLOCK = 1 << 24


class LatticeQMC:

    def __init__(self, model, beta, time_steps, warmup=300, sweeps=2000, det_mode=False,
                 log_lvl=DEBUG, *, mode=None, precision="fp64", rng=None, stab_every=None,
                 seed=0, device=0, delay=0, engine="auto", fp64e_native=("lu", "lu_rhs"),
                 measure_tau=False):
        self.logger = _log if log_lvl is not None else None
        if self.logger is not None:
            self.logger.setLevel(log_lvl)
        self.model = model
        self.n_sites = model.n_sites
        self.time_steps = time_steps
        self.config = Configuration(self.n_sites, time_steps)
        self.warm_sweeps = warmup
        self.meas_sweeps = sweeps
        self.det_mode = det_mode
        self.mode = mode or ("dqmc" if det_mode else "compat")
        self.precision = precision
        self.rng = rng or "replay"
        self.stab_every = stab_every
        self.seed = seed
        self.device = device
        self.delay = delay
        self.engine_kind = engine
        self.fp64e_native = fp64e_native
        self.measure_tau = bool(measure_tau)
        self.status = ""
        self.it = 0
        self.ratio = 0.0
        self.acc = False
        self.ham_kin = self.model.ham_kinetic()
        self.beta = 0.
        self.dtau = 0.
        self.lamb = 0.
        self.exp_k = None
        self._engine = None
        self._engine_det = None
        self._log_info(f"Warmup=     {self.warm_sweeps}")
        self._log_info(f"Measurement={self.meas_sweeps}")
        self.set_beta(beta)

    def _log_info(self, msg):
        if self.logger is not None:
            self.logger.info(msg)

    def set_beta(self, beta):
        """dtau, lambda and exp_k as lqmc.py:93-117; the device chain is (re)built lazily."""
        self.dtau = beta / self.time_steps
        self.beta = beta
        self.lamb = hs_coupling(self.model.u, self.dtau)
        self._engine = None
        self._engine_det = None
        spec = ChainSpec(self.ham_kin, self.model.u, beta, self.time_steps, self.config.config)
        self.exp_k = spec.exp_k
        self._spec = spec

    def set_temperature(self, temp):
        self.set_beta(1 / temp)

    @property
    def engine(self):
        if self._engine is None:
            self._engine = Engine([self._spec], mode=self.mode, precision=self.precision,
                                  rng=self.rng, stab_every=self.stab_every, seed=self.seed,
                                  device=self.device, delay=self.delay, engine=self.engine_kind,
                                  fp64e_native=self.fp64e_native, measure_tau=self.measure_tau)
        return self._engine

    def _det_engine(self):
        """The device engine of the reference's determinant mode (mode 'det', float64)."""
        if self._engine_det is None:
            self._engine_det = Engine([self._spec], mode="det", precision="fp64", rng=self.rng,
                                      stab_every=self.stab_every, seed=self.seed,
                                      device=self.device)
        return self._engine_det

    def iter_sweeps(self, n, console_updates=200):
        """Yield 0 .. n-1 with ``self.it`` set and a progress line on the console every
        n / console_updates sweeps, as lqmc.py:187-215."""
        every = max(1, int(n / console_updates))
        for it in range(n):
            if (it + 1) % every == 0:
                print(f"\r{self.status} Sweep {it + 1} ({100 * (it + 1) / n:.1f}%) "
                      f"[Mean: {self.config.mean():5.2f}, Var: {self.config.var():5.2f}]",
                      end="", flush=True)
            self.it = it
            yield it
        print(f"\r{self.status} Sweep {n} (100.0%)")

    # -- sweeps ----------------------------------------------------------------------------
    def _run(self, n_sweeps, measure, eng=None):
        eng = eng if eng is not None else self.engine
        eng.set_field(0, self.config.config)
        per = self.n_sites * self.time_steps
        done = 0
        while done < n_sweeps:
            k = n_sweeps - done
            if self.rng == "replay":
                k = max(1, min(k, _REPLAY_BLOCK // per))
                eng.set_uniforms(0, np.random.rand(k * per))
            eng.sweep(k, measure=measure)
            done += k
        self.config.config = eng.field(0)

    def _update_step(self):
        """One sweep (lqmc.py:301-347); returns (G_up, G_dn) after slice 0."""
        self._run(1, False)
        g = self.engine.green(0)
        return g[0], g[1]

    def warmup_loop(self):
        self.status = "Warmup"
        self._run(self.warm_sweeps, False)

    def measure_loop(self):
        """Mean of the end-of-sweep G over the measurement sweeps (lqmc.py:356-375)."""
        self.status = "Measurement"
        self.engine.reset_measurements()
        self._run(self.meas_sweeps, True)
        gsum, cnt = self.engine.green_sum(0)
        return gsum / max(cnt, 1)

    # -- the reference's determinant mode (lqmc.py:236-299), on the device ---------------------
    def _update_step_det(self, old_det=None):
        """One determinant-mode sweep (lqmc.py:236-259): every flip's ratio is
        det M_up det M_dn of the flipped field over the current one.  Returns that product for
        the field the sweep leaves, as the reference returns its running old_det (which is
        always a fresh determinant).  ``old_det`` is taken for the reference's signature; the
        device computes it from the field."""
        eng = self._det_engine()
        self._run(1, False, eng)
        d = eng.diagnostics(0)
        # the kernel keeps log|det G_sigma| = -log|det M_sigma| and sign(det M_sigma)
        return float(np.prod(d["sign"]) * np.exp(-np.sum(d["logdet"])))

    def warmup_loop_det(self):
        """Warm-up sweeps of the determinant mode (lqmc.py:261-271)."""
        self.status = "Warmup"
        self._run(self.warm_sweeps, False, self._det_engine())

    def measure_loop_det(self):
        """Mean of inv(get_m(0, sigma)) over the determinant-mode measurement sweeps
        (lqmc.py:273-299)."""
        self.status = "Measurement"
        eng = self._det_engine()
        eng.reset_measurements()
        self._run(self.meas_sweeps, True, eng)
        gsum, cnt = eng.green_sum(0)
        return gsum / max(cnt, 1)

    def observables(self):
        """Wick observables averaged over the last measurement loop."""
        return self.engine.observables(0)

    def green_tau(self):
        """Mean unequal-time G_sigma(tau_l, 0), l = 0 .. L-1, over the last measurement loop,
        shape (2, L, N, N) (measure_tau=True); minus lqmc.tools.compute_pole_gf_tau's G(tau)
        at U = 0."""
        if not self.measure_tau:
            raise ValueError("green_tau needs LatticeQMC(..., measure_tau=True)")
        return self.engine.green_tau(0)

    def run_lqmc(self):
        self.warmup_loop()
        return self.measure_loop()

    def run(self):
        t0 = time.time()
        gf_tau = self.run_lqmc()
        t = time.time() - t0
        mins, secs = divmod(t, 60)
        self._log_info(f"Total time: {int(mins):0>2}:{int(secs):0>2} min")
        return gf_tau
