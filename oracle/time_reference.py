"""Time the reference's own fast sweep (lqmc/lqmc.py:301-347) against the CPU port that the
bench reports as its baseline (oracle/compat.py), on one core with one BLAS thread.

Test infrastructure, not product: it imports the reference from the directory named by the
LQMC_REFERENCE environment variable (required), so it runs only where the reference is present.

Workload: periodic 16x16 square lattice, t = 1, U = 4, mu = 0, dtau = 0.1. The reference's
lattice builder cannot close a 16x16 periodic lattice (lqmc/lattice.py:1030-1031), so a
stand-in model object hands it the kinetic matrix of this package's builder. That builder
equals the reference's on every size the reference can build.

Both codes sweep the same field with the same uniform stream, so their accept/reject decisions
are the same. A sweep of L = 4 slices (1024 site updates; the one-off from-scratch G and the
three wraps are ~1 % of it) is timed for each code, alternating the order over three
repetitions; the medians are reported.

    OPENBLAS_NUM_THREADS=1 python -m oracle.time_reference
"""
import os
import sys
import time
import types

import numpy as np

REF = os.environ.get("LQMC_REFERENCE")
if not REF:
    raise SystemExit("set LQMC_REFERENCE to the directory that holds the reference's lqmc package")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _import_reference():
    # the reference imports matplotlib at module top only for plotting
    for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.collections", "mpl_toolkits",
                 "mpl_toolkits.axes_grid1"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["matplotlib.collections"].LineCollection = object
    sys.modules["mpl_toolkits.axes_grid1"].make_axes_locatable = None
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    sys.path.insert(0, REF)
    from lqmc import LatticeQMC
    return LatticeQMC


class _Model:
    """The attributes LatticeQMC reads from its model (lqmc/lqmc.py:48-112)."""

    def __init__(self, kinetic, u, t=1.0, mu=0.0):
        self.n_sites = kinetic.shape[0]
        self._k = kinetic
        self.u, self.t, self.mu = u, t, mu

    def ham_kinetic(self):
        return self._k.copy()


def time_pair(LatticeQMC, kinetic, u, dtau, L, seed, port_first):
    """Seconds of one reference sweep and one port sweep of L slices, same field and stream."""
    from oracle import compat
    np.random.seed(seed)
    ref = LatticeQMC(_Model(kinetic, u), dtau * L, L, warmup=0, sweeps=0, log_lvl=None)
    field0 = ref.config.config.copy()
    state = np.random.get_state()
    uni = np.random.rand(field0.size)
    np.random.set_state(state)
    field = field0.copy()

    def run_port():
        t0 = time.perf_counter()
        compat.update_step(ref.exp_k, field, ref.lamb, uni, rank1="loop", log_line=True)
        return time.perf_counter() - t0

    def run_ref():
        t0 = time.perf_counter()
        ref._update_step()
        return time.perf_counter() - t0

    if port_first:
        t_port = run_port()
        t_ref = run_ref()
    else:
        t_ref = run_ref()
        t_port = run_port()
    assert np.array_equal(field, ref.config.config), "the port's decisions differ"
    return t_ref, t_port


def main(side=16, u=4.0, dtau=0.1, seed=7):
    sys.path.insert(0, ROOT)
    from latticeqmc_gb300 import HubbardModel
    LatticeQMC = _import_reference()
    m = HubbardModel(u=u, t=1, mu=0)
    m.build_square(side)
    kinetic = m.ham_kinetic()
    n = side * side
    L = 4
    times = [time_pair(LatticeQMC, kinetic, u, dtau, L, seed + rep, port_first=rep % 2 == 0)
             for rep in range(3)]
    ref_site = float(np.median([t[0] for t in times])) / (n * L)
    port_site = float(np.median([t[1] for t in times])) / (n * L)
    print(f"{side}x{side}, U={u}, dtau={dtau}, L={L}, one process, medians of 3: reference "
          f"{1 / ref_site:.1f} site-updates/s, port {1 / port_site:.1f} site-updates/s, "
          f"port / reference {ref_site / port_site:.2f}; per repetition (reference s, port s): "
          + ", ".join(f"({a:.1f}, {b:.1f})" for a, b in times))


if __name__ == "__main__":
    main()
