"""Batched Markov-chain engine over liblqmc_gpu.so.

One ``Engine`` holds any number of independent chains (uneven lattice sizes, temperatures
and interactions allowed) and sweeps them all in one launch per shared-memory footprint.
It replaces the reference's walker pool (lqmc/multiprocessing.py:252-341), which ran one
chain per forked process.

Host-side set-up follows ``LatticeQMC.set_beta`` (lqmc/lqmc.py:93-117) with the same numpy /
scipy call forms, so the float64 constants handed to the device are bit-identical to the
ones the reference computes:
    dtau = beta / L;  lambda = arccosh(exp(U dtau / 2)) (0 if U == 0);  exp_k = expm(-dtau K)
"""
import ctypes

import numpy as np
from scipy.linalg import expm

from . import _native
from ._native import as_f64, ptr


def hs_coupling(u, dtau):
    """lambda = arccosh(exp(U dtau / 2)), or 0 for U == 0 (lqmc/lqmc.py:105)."""
    return np.arccosh(np.exp(u * dtau / 2.)) if u else 0


def exp_constants(lamb, n_sites):
    """[exp(2 lam), exp(-2 lam), exp(-lam), exp(lam)] in the reference's call forms.

    exp(+-2 lam) are numpy scalar exps of arg = 2 * lamb * s (lqmc/lqmc.py:313-323);
    exp(-+lam) come from numpy's array exp over an int8 field column (lqmc/lqmc.py:149-154).
    """
    e2p = np.exp(+(2 * lamb * np.int8(1)))
    e2m = np.exp(+(2 * lamb * np.int8(-1)))
    col = np.array(([1, -1] * ((n_sites + 2) // 2))[:max(n_sites, 2)], dtype=np.int8)
    ev = np.exp(-1 * 1 * lamb * col)
    return np.array([e2p, e2m, ev[0], ev[1]], dtype=np.float64)


def auto_stab_every(chains):
    """Slices between refreshes of G: the largest n_s with n_s * dtau <= 0.5 for every chain.

    The wraps between refreshes amplify rounding by up to exp(n_s dtau (8t + 2 lambda)); at
    n_s dtau <= 0.5 the float64 G stays within ~1e-12 of a fresh recompute."""
    return max(1, min(int(0.5 / c.dtau + 1e-9) for c in chains))


class ChainSpec:
    """One chain: kinetic matrix K (N, N), interaction u, inverse temperature beta,
    time slices L and the initial HS field (N, L) int8.

    exp_k, exp_k_inv and consts may be given precomputed (e.g. values recorded on another
    machine); otherwise they are computed here as the reference does."""

    def __init__(self, kinetic, u, beta, time_steps, field, exp_k=None, exp_k_inv=None,
                 consts=None):
        self.kinetic = as_f64(kinetic)
        self.n = self.kinetic.shape[0]
        self.u = float(u)
        self.beta = float(beta)
        self.L = int(time_steps)
        self.field = np.ascontiguousarray(field, dtype=np.int8)
        if self.field.shape != (self.n, self.L):
            raise ValueError(f"field shape {self.field.shape} != ({self.n}, {self.L})")
        self.dtau = self.beta / self.L
        self.lamb = hs_coupling(u, self.dtau)
        self.exp_k = as_f64(exp_k) if exp_k is not None else expm(-1 * self.dtau * self.kinetic)
        self.exp_k_inv = None if exp_k_inv is None else as_f64(exp_k_inv)
        self.consts = None if consts is None else as_f64(consts)


class Engine:
    """Batched DQMC sweep engine on one GPU.

    mode       'compat' (reference arithmetic, lqmc/lqmc.py:301-347), 'dqmc' (textbook,
               stabilised) or 'det' (the reference's determinant mode, lqmc/lqmc.py:236-299:
               every ratio from det M of the flipped configuration; a slow check path)
    precision  'fp64'; 'fp64e' (float64 G and updates, every dense product a float64-accurate
               GEMM emulated on the BF16 tensor cores); or 'mixed' (float32 G, wraps, updates
               and B-chain products; float64 Householder QR and LU of the stabilisation)
    rng        'replay' (uniforms uploaded per sweep) or 'philox' (on device)
    engine     'auto', 'smem' (one CTA per chain, G in shared memory, fp64, N <= 128) or
               'tiled' (matrices in global memory, tiled GEMMs; any N up to 2048)
    fp64e_native  product categories the fp64e engine keeps in native float64: names from
               'wrap', 'stack', 'udt', 'green', 'update', 'lu', 'lu_rhs' (or an
               LQMC_FP64E_NATIVE_* mask).  Default ('lu', 'lu_rhs'): the stabilised inverse's LU
               solve in float64 (emulating its right-hand-side updates is ~5 % faster at 16x16,
               beta=8, but leaves a 7x larger median stabilisation residual)
    measure_tau  also accumulate the unequal-time G(tau_l, 0) of every slice on each measured
               sweep ('dqmc' only; a float64 kernel per sweep after the sweep kernel; read with
               green_tau / green_tau_sum)
    sweep_order  'down' (every sweep l = L-1 .. 0, the reference's order) or 'alternate'
               ('dqmc' only, tiled kernel: sweeps alternate down and up, so each direction's
               UDT products serve the next sweep instead of a from-scratch rebuild; decisions
               are recorded in visit order; a checkpoint resumes with a rebuild, equal to the
               uninterrupted run only to rounding)
    oz_stages  'fp64e': stage buffers of the emulated GEMM's copy / MMA ring (1 .. 3; 0: the
               engine's rule)
    """

    def __init__(self, chains, mode="dqmc", precision="fp64", rng="philox", stab_every=None,
                 delay=0, seed=0, record=False, device=0, engine="auto", debug=0,
                 fp64e_native=("lu", "lu_rhs"), measure_tau=False, sweep_order="down",
                 oz_stages=0):
        self.chains = list(chains)
        if stab_every is None:
            stab_every = auto_stab_every(self.chains)
        self.stab_every = int(stab_every)
        self.mode, self.precision, self.rng = mode, precision, rng
        self.record = bool(record)
        self.measure_tau = bool(measure_tau)
        self.sweep_order = sweep_order
        self._h = _native.Handle(mode, precision, rng, stab_every, delay, seed, record, device,
                                 engine, debug, fp64e_native, measure_tau, sweep_order, oz_stages)
        n = len(self.chains)
        n_sites = np.array([c.n for c in self.chains], dtype=np.int32)
        n_slices = np.array([c.L for c in self.chains], dtype=np.int32)
        eks, ekis, kins = [], [], []
        consts = np.zeros((n, 4))
        us = np.zeros(n)
        for i, c in enumerate(self.chains):
            eks.append(as_f64(c.exp_k))
            if c.exp_k_inv is not None:
                ekis.append(c.exp_k_inv)
            elif mode == "compat":
                ekis.append(as_f64(np.linalg.inv(c.exp_k)))
            else:
                ekis.append(as_f64(expm(c.dtau * c.kinetic)))
            kins.append(c.kinetic)
            consts[i] = c.consts if c.consts is not None else exp_constants(c.lamb, c.n)
            us[i] = c.u
        self._keep = (eks, ekis, kins)
        arr = ctypes.c_void_p * n
        p_ek = arr(*[m.ctypes.data for m in eks])
        p_eki = arr(*[m.ctypes.data for m in ekis])
        p_kin = arr(*[m.ctypes.data for m in kins])
        self._h.call("lqmc_set_chains", n, ptr(n_sites), ptr(n_slices), p_ek, p_eki, p_kin,
                     ptr(consts), ptr(us))
        for i, c in enumerate(self.chains):
            self.set_field(i, c.field)
        self.last_sweeps = 0

    # -- state ---------------------------------------------------------------------------
    def set_field(self, chain, field):
        f = np.ascontiguousarray(field, dtype=np.int8)
        self._h.call("lqmc_set_field", int(chain), ptr(f))

    def field(self, chain):
        c = self.chains[chain]
        out = np.empty((c.n, c.L), dtype=np.int8)
        self._h.call("lqmc_get_field", int(chain), ptr(out))
        return out

    def set_uniforms(self, chain, uniforms):
        u = as_f64(uniforms)
        self._h.call("lqmc_set_uniforms", int(chain), ptr(u), u.size)

    def set_uniforms_all(self, uniforms):
        """Uniforms of every chain in one copy: concatenation over chains of
        (n_sweeps, N*L) blocks.  `uniforms` may be pinned host memory (a numpy view)."""
        u = as_f64(uniforms)
        self._h.call("lqmc_set_uniforms_all", ptr(u), u.size)

    # -- sweeps --------------------------------------------------------------------------
    def sweep(self, n_sweeps=1, measure=False, stream=None):
        """Run n_sweeps sweeps of every chain (asynchronous on `stream`, an int handle)."""
        self._h.call("lqmc_sweep", int(n_sweeps), int(bool(measure)),
                     ctypes.c_void_p(stream or 0))
        self.last_sweeps = int(n_sweeps)

    # -- results -------------------------------------------------------------------------
    def green(self, chain):
        c = self.chains[chain]
        out = np.empty((2, c.n, c.n))
        self._h.call("lqmc_get_green", int(chain), ptr(out))
        return out

    def green_all(self, out=None):
        """G of every chain, concatenated (sum of 2 N^2 doubles), in one copy."""
        total = sum(2 * c.n * c.n for c in self.chains)
        if out is None:
            out = np.empty(total)
        self._h.call("lqmc_get_green_all", ptr(out))
        return out

    def green_sum(self, chain):
        c = self.chains[chain]
        out = np.empty((2, c.n, c.n))
        cnt = np.zeros(1, dtype=np.int64)
        self._h.call("lqmc_get_green_sum", int(chain), ptr(out), ptr(cnt))
        return out, int(cnt[0])

    def green_tau_sum(self, chain):
        """Sum over the measured sweeps of G_sigma(tau_l, 0) = <c_i(tau_l) c+_j(0)>,
        tau_l = l dtau, l = 0 .. L-1, shape (2, L, N, N), and the measurement count
        (measure_tau=True): B(tau_l, 0) (1 + B(beta, 0))^-1 with B_l = exp_v(l) exp_k.
        G(tau, 0) is minus lqmc.tools.compute_pole_gf_tau's G(tau) at U = 0.  The end-of-sweep
        G that green_sum adds up is the equal-time G at tau_1: per sample
        G(tau_1, 0) = G_sweep B_0."""
        c = self.chains[chain]
        out = np.empty((2, c.L, c.n, c.n))
        self._h.call("lqmc_get_green_tau", int(chain), ptr(out))
        return out, int(self.observables_raw(chain)[0])

    def green_tau(self, chain):
        """Mean G_sigma(tau_l, 0) over the measured sweeps, shape (2, L, N, N)."""
        s, cnt = self.green_tau_sum(chain)
        return s / max(cnt, 1)

    def observables_raw(self, chain):
        c = self.chains[chain]
        out = np.empty(_native.obs_len(c.n))
        self._h.call("lqmc_get_observables", int(chain), ptr(out))
        return out

    def observables(self, chain):
        """Means over the measured sweeps of chain `chain` (dict)."""
        n = self.chains[chain].n
        o = self.observables_raw(chain)
        cnt = max(o[0], 1.0)
        h = _native.OBS_HEADER
        return {
            "count": int(o[0]),
            "kinetic_energy": o[1] / cnt,
            "potential_energy": o[2] / cnt,
            "double_occupancy_mean": o[3] / cnt,
            "density_mean": o[4] / cnt,
            "density": o[h:h + n] / cnt,
            "double_occupancy": o[h + n:h + 2 * n] / cnt,
            "nn": o[h + 2 * n:h + 2 * n + n * n].reshape(n, n) / cnt,
            "szsz": o[h + 2 * n + n * n:h + 2 * n + 2 * n * n].reshape(n, n) / cnt,
        }

    def set_measurement_sums(self, chain, green_sum, obs):
        """Overwrite a chain's sum of G (2, N, N) and its observable sums (the count in
        obs[0] included), e.g. to drop measurements taken after its share of sweeps."""
        g = as_f64(green_sum)
        o = as_f64(obs)
        self._h.call("lqmc_set_chain_state", int(chain), None, ptr(g), ptr(o))

    def reset_measurements(self):
        self._h.call("lqmc_reset_measurements")

    def decisions(self, chain):
        c = self.chains[chain]
        out = np.empty((self.last_sweeps, c.L, c.n), dtype=np.int8)
        self._h.call("lqmc_get_decisions", int(chain), ptr(out), out.size)
        return out

    def diagnostics(self, chain):
        d = np.empty(_native.DIAG_LEN)
        self._h.call("lqmc_get_diagnostics", int(chain), ptr(d))
        return {"accepted": d[0], "attempted": d[1], "max_residual": d[2],
                "logdet": d[3:5].copy(), "sign": d[5:7].copy(), "sweeps": int(d[7]),
                "phase_cycles": {"recompute": d[8], "update": d[9], "wrap": d[10],
                                 "stabilise": d[11], "measure": d[12]},
                "sub_cycles": {"qr": d[13], "q_and_t": d[14], "lu": d[15],
                               "oz_split": d[16], "oz_mma": d[17], "oz_epilogue": d[18],
                               "flush": d[19], "site_barrier": d[20]}}

    # -- checkpoint / resume -------------------------------------------------------------
    def checkpoint(self, path):
        """Write every chain's state (field, diagnostics with the Philox sweep counter, sum of
        G, observable sums) and the engine's settings to an .npz file."""
        arrays = {"n_sites": np.array([c.n for c in self.chains]),
                  "n_slices": np.array([c.L for c in self.chains]),
                  "settings": np.array([self.mode, self.precision, self.rng, str(self.stab_every)])}
        for k in range(len(self.chains)):
            d = np.empty(_native.DIAG_LEN)
            self._h.call("lqmc_get_diagnostics", int(k), ptr(d))
            gsum, _ = self.green_sum(k)
            arrays[f"field_{k}"] = self.field(k)
            arrays[f"diag_{k}"] = d
            arrays[f"gsum_{k}"] = gsum
            arrays[f"obs_{k}"] = self.observables_raw(k)
            if self.measure_tau:
                arrays[f"gtau_{k}"] = self.green_tau_sum(k)[0]
        np.savez(path, **arrays)

    def restore(self, path):
        """Resume from a checkpoint of an engine with the same chains and settings (the seed
        is not stored: pass the same seed to the new Engine)."""
        z = np.load(path)
        if (list(z["n_sites"]) != [c.n for c in self.chains]
                or list(z["n_slices"]) != [c.L for c in self.chains]):
            raise ValueError("checkpoint was written for different chains")
        want = [self.mode, self.precision, self.rng, str(self.stab_every)]
        if list(z["settings"]) != want:
            raise ValueError(f"checkpoint settings {list(z['settings'])} differ from {want}")
        for k in range(len(self.chains)):
            self.set_field(k, z[f"field_{k}"])
            d = np.ascontiguousarray(z[f"diag_{k}"], dtype=np.float64)
            g = np.ascontiguousarray(z[f"gsum_{k}"], dtype=np.float64)
            o = np.ascontiguousarray(z[f"obs_{k}"], dtype=np.float64)
            self._h.call("lqmc_set_chain_state", int(k), ptr(d), ptr(g), ptr(o))
            if self.measure_tau:
                if f"gtau_{k}" not in z:
                    raise ValueError("checkpoint holds no unequal-time G sums")
                gt = np.ascontiguousarray(z[f"gtau_{k}"], dtype=np.float64)
                self._h.call("lqmc_set_green_tau", int(k), ptr(gt))

    def status(self):
        s = np.empty(len(self.chains), dtype=np.int32)
        self._h.check(self._h.lib.lqmc_get_status(self._h.h, ptr(s)))
        return s

    def launch_count(self):
        v = np.zeros(1, dtype=np.int64)
        self._h.check(self._h.lib.lqmc_get_launch_count(self._h.h, ptr(v)))
        return int(v[0])

    def close(self):
        self._h.close()
