"""Run one sweep configuration and print its timing and per-phase split.

    python -m latticeqmc_gb300.runcase --side 16 --beta 1.6 --L 16 --precision fp64e \
        --chains 1 --sweeps 1

Used to profile a single kernel launch on a small case: one lqmc_sweep call of `--sweeps`
sweeps of every chain (periodic square lattice, t=1, mu=0, dqmc mode, Philox uniforms).
"""
import argparse
import time

import numpy as np

from . import ChainSpec, Engine, HubbardModel


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--side", type=int, default=16)
    ap.add_argument("--u", type=float, default=4.0)
    ap.add_argument("--beta", type=float, default=8.0)
    ap.add_argument("--L", type=int, default=80)
    ap.add_argument("--stab", type=int, default=8)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp64e", "mixed"])
    ap.add_argument("--engine", default="auto", choices=["auto", "smem", "tiled"])
    ap.add_argument("--chains", type=int, default=1)
    ap.add_argument("--sweeps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=0)
    ap.add_argument("--delay", type=int, default=0, help="delayed-update depth (0: automatic)")
    a = ap.parse_args()
    m = HubbardModel(u=a.u, t=1, mu=0)
    m.build_square(a.side)
    K = m.ham_kinetic()
    n = a.side * a.side
    rng = np.random.default_rng(0)
    specs = [ChainSpec(K, a.u, a.beta, a.L, (2 * rng.integers(0, 2, (n, a.L)) - 1).astype(np.int8))
             for _ in range(a.chains)]
    eng = Engine(specs, mode="dqmc", precision=a.precision, rng="philox", seed=1,
                 stab_every=a.stab, engine=a.engine, delay=a.delay)
    if a.warmup:
        eng.sweep(a.warmup)
        eng.green(0)
    t0 = time.perf_counter()
    eng.sweep(a.sweeps)
    eng.green(0)
    dt = time.perf_counter() - t0
    d = eng.diagnostics(0)
    pc = d["phase_cycles"]
    tot = max(sum(pc.values()), 1.0)
    print(f"{a.side}x{a.side} L={a.L} {a.precision} chains={a.chains} delay={a.delay or 'auto'}: "
          f"{dt * 1e3 / a.sweeps:.1f} ms/sweep, residual {d['max_residual']:.1e}, "
          + " ".join(f"{k}={100 * v / tot:.1f}%" for k, v in pc.items()) + " | "
          + " ".join(f"{k}={100 * v / tot:.1f}%" for k, v in d["sub_cycles"].items()))
    eng.close()


if __name__ == "__main__":
    main()
