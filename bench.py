"""Throughput benchmark of the DQMC sweep engine on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload square16_beta8 | batched_fp64 | square32_beta6]

A step is one sweep of every chain of the workload (one lqmc_sweep(1) call).  The metric
is site-updates/s: sum over chains of N_c * L_c site-update attempts per sweep, divided by
the time per sweep; sweeps/s is reported beside it.  Inputs are synthetic random HS fields
(the reference's own runs start from random fields), t=1, mu=0, periodic square lattices.

Workload square16_beta8 (default; the configuration the metric "batched mixed vs plain
FP64 at max|dG| <= 1e-6" is quoted on): 64 chains of 16x16 (N=256), U=4, beta=8, dtau=0.1
(L=80), dqmc, on-device Philox uniforms; stabilisation interval, sweep order, delay depth,
stage count and native-float64 categories of the headline engine from the project
autotuner's record for this shape (latticeqmc_gb300/tuning/autotune.json; stab_every within
6-16, see STAB_RANGE), else stabilisation every 8 slices in the alternating order.  `value`
is the batched mixed-precision engine that meets the max|dG| <= 1e-6 bar: precision "fp64e",
every dense product (wraps, B-chain, delayed rank-k updates, the blocked QR's and the LU's
updates) a float64-accurate GEMM emulated on the tcgen05 BF16 tensor cores, the per-site
updates and the panel factorisations in float64.  `fp64` carries the plain float64 engine
on the same workload, stabilisation interval and sweep order (throughput and the speed-up of
`value` over it) and `fp32_mixed` the float32 engine; `accuracy` compares fp64e with fp64
over several sweeps from identical fields and uniforms; `tuning` names the chosen setting
and the runner-up.  Time-bounded sub-records of the other workloads ride on the same line:
`batched_fp64` (512 uneven chains against the same chains run one at a time) and
`square32_beta6` (32x32 chains, fp64e).

Workload batched_fp64: 512 chains, 128 each of 4x4, 6x6, 8x8, 10x10, U drawn per chain
from {2, 4, 6}, beta=4, L=40, dqmc float64, stabilisation every 5 slices.
Workload square32_beta6: 32x32 (N=1024), U=4, beta=6, L=60, dqmc fp64e, stabilisation every
5 slices (the engine's stab_every * dtau <= 0.5 rule: at 10, 40 of 76 chains drifted past the
1e-6 residual bar, at 6 one did), alternating sweep order, one chain per pair of SMs (one
wave); the chain count HBM would admit is reported.

value      device throughput with all state resident in HBM.
e2e        the same sweeps through the public C ABI in replay mode (the drop-in path of
           LatticeQMC._update_step): each step uploads that sweep's uniforms from pinned
           host memory and downloads every chain's G, copies inside the timed region.
roofline   algorithmic float64 flops per sweep and chain
           F = 8 L N^3 (wraps) + 4 L N^3 (B-chain) + 2 (L / n_s) (4/3) N^3 (QR) + 4 A N^2
           (A = accepted flips, counted on the device).  fp64e engine: bound "tensor",
           achieved = 36 F / sweep time (each float64 product is 36 BF16 slice products),
           peak = the measured sustained BF16 rate (MEASURED_PEAKS.json); `fp64_equivalent`
           gives F / time against the float64 DGEMM rate measured here.  batched_fp64
           workload: F / time against that DGEMM rate.
cpu_baseline  the reference's fast sweep restated in Python/numpy (oracle/compat.py, with
           the pure-Python rank-1 loop of lqmc.py:328-331) on a bounded sample of every
           lattice size of the workload, one process per host core; `single_process`
           gives the same on one core.

With --gpus N > 1 and no launcher environment, bench.py starts N ranks itself through
torch.distributed.run (127.0.0.1); under a launcher, WORLD_SIZE must equal N.
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import socket
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "site-updates/s (sweeps/s beside it), DQMC sweep of batched Markov chains"
UNIT = "site-updates/s"
# DRAM traffic of one fp64e sweep launch of the square16_beta8 workload (64 chains, the tuned
# settings), from ncu: dram__bytes_read.sum + dram__bytes_write.sum, mean of 2 launches
FP64E_TRAFFIC = 2.774e11
STATUS_BITS = {"nonfinite": 1, "singular": 2, "drift": 4, "timeout": 8}


# ----------------------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------------------
def workload_batched(rank=0, per_side=128):
    from latticeqmc_gb300 import ChainSpec, HubbardModel
    sides = [4, 6, 8, 10]
    beta, L = 4.0, 40
    rng = np.random.default_rng(1000 + rank)
    specs = []
    kin = {}
    for side in sides:
        m = HubbardModel(u=4, t=1, mu=0)
        m.build_square(side)
        kin[side] = m.ham_kinetic()
    for side in sides:
        for _ in range(per_side):
            u = float(rng.choice([2.0, 4.0, 6.0]))
            n = side * side
            field = (2 * rng.integers(0, 2, (n, L)) - 1).astype(np.int8)
            specs.append(ChainSpec(kin[side], u, beta, L, field))
    cfg = {"workload": f"batched_fp64: {4 * per_side} chains = {per_side} x {{4x4, 6x6, 8x8, 10x10}} periodic, "
                       "U in {2,4,6} per chain, mu=0, beta=4, dtau=0.1 (L=40), dqmc fp64, "
                       "stab every 5, philox",
           "chains": len(specs), "sides": sides, "beta": beta, "L": L, "stab_every": 5,
           "precision": "fp64", "mode": "dqmc"}
    return specs, cfg


def workload_square(rank=0, chains=64, side=16, beta=8.0, L=80, stab=8, name="square16_beta8",
                    precision="fp64e (value); fp64 and fp32 mixed reported beside it"):
    from latticeqmc_gb300 import ChainSpec, HubbardModel
    u = 4.0
    m = HubbardModel(u=u, t=1, mu=0)
    m.build_square(side)
    kin = m.ham_kinetic()
    rng = np.random.default_rng(2000 + rank + 7919 * side)
    n = side * side
    specs = [ChainSpec(kin, u, beta, L, (2 * rng.integers(0, 2, (n, L)) - 1).astype(np.int8))
             for _ in range(chains)]
    cfg = {"workload": f"{name}: {chains} chains of {side}x{side} periodic (N={n}), U=4, mu=0, "
                       f"beta={beta:g}, dtau={beta / L:g} (L={L}), dqmc, stab every {stab}, philox",
           "chains": chains, "sides": [side], "beta": beta, "L": L, "stab_every": stab,
           "precision": precision, "mode": "dqmc"}
    return specs, cfg


def workload_square16(rank=0, chains=64):
    return workload_square(rank, chains)


def algorithmic_flops(specs, accepted, stab_every):
    tot = 0.0
    for c in specs:
        n, L = c.n, c.L
        tot += 8.0 * L * n ** 3 + 4.0 * L * n ** 3 + 2.0 * math.ceil(L / stab_every) * (4.0 / 3.0) * n ** 3
    return tot + sum(4.0 * a * c.n ** 2 for a, c in zip(accepted, specs))


def config_extras(world):
    """Keys both arms add to the workload's config."""
    return {"parallelism": f"chains sharded over {world} GPU(s)",
            "l2": "working set (per-chain G, GEMM temporaries and UDT stacks; 0.6-1.6 GB) "
                  "exceeds the 129 MB L2; no flush"}


# ----------------------------------------------------------------------------------------
# clocks
# ----------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------------------
# CPU baseline (the reference's algorithm, oracle port)
# ----------------------------------------------------------------------------------------
def _cpu_worker(args):
    side, L, beta, u, seconds, seed = args
    sys.path.insert(0, ROOT)
    from oracle import compat
    from latticeqmc_gb300 import HubbardModel
    from latticeqmc_gb300.engine import ChainSpec
    m = HubbardModel(u=u, t=1, mu=0)
    m.build_square(side)
    n = side * side
    rng = np.random.default_rng(seed)
    field = (2 * rng.integers(0, 2, (n, L)) - 1).astype(np.int8)
    spec = ChainSpec(m.ham_kinetic(), u, beta, L, field)
    uni = rng.random(n * L)
    # size the sample from a short probe so that it takes about `seconds`; the per-site
    # cost is the slope between a sample and one twice as long, which removes the one-off
    # from-scratch G at the start of the sweep
    probe = compat.time_sites(spec.exp_k, field.copy(), spec.lamb, uni, min(n * L, 16))
    s1 = int(min(n * L // 2, max(8, seconds / 3.0 / max(probe, 1e-9))))
    t1 = compat.time_sites(spec.exp_k, field.copy(), spec.lamb, uni, s1) * s1
    t2 = compat.time_sites(spec.exp_k, field.copy(), spec.lamb, uni, 2 * s1) * 2 * s1
    return side, max(t2 - t1, 1e-9) / s1, 3 * s1


def cpu_baseline(specs, cfg, seconds_per_size=2.5, cores=None):
    """Site-updates/s of the workload on `cores` host processes, each running a bounded
    sample of the reference's sweep for every lattice size."""
    cores = cores or os.cpu_count() or 1
    sides = cfg["sides"]
    jobs = []
    for p in range(cores):
        for side in sides:
            jobs.append((side, cfg["L"], cfg["beta"], 4.0, seconds_per_size, 7 + p))
    ctx = mp.get_context("spawn")
    # one BLAS thread per process: the children read this when they import numpy
    saved = {k: os.environ.get(k) for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS")}
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"
    t0 = time.perf_counter()
    try:
        with ctx.Pool(cores) as pool:
            res = pool.map(_cpu_worker, jobs)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    wall = time.perf_counter() - t0
    t_site = {s: statistics.mean(r[1] for r in res if r[0] == s) for s in sides}
    samples = {s: sum(r[2] for r in res if r[0] == s) for s in sides}
    # one batch sweep = every chain's N L site updates; chains spread over the cores
    serial = sum(c.n * c.L * t_site[int(round(math.sqrt(c.n)))] for c in specs)
    per_sweep = serial / cores
    sites = sum(c.n * c.L for c in specs)
    return {
        "value": sites / per_sweep,
        "unit": UNIT,
        "cores": cores,
        "kind": "port",
        "sample": (f"oracle/compat.py fast sweep (pure-Python rank-1 loop, per-site log line), "
                   f"{', '.join(f'{s}x{s}: {samples[s]} site updates' for s in sides)} over "
                   f"{cores} processes, {wall:.1f}s wall; extrapolated to one sweep of all "
                   f"{len(specs)} chains"),
        "sweep_seconds": per_sweep,
        "wall_seconds": wall,
    }


# ----------------------------------------------------------------------------------------
# GPU measurement
# ----------------------------------------------------------------------------------------
def fp64_peak_tflops(torch):
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = max(best, 2.0 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    return best


def status_counts(status):
    """Chains with each LQMC_STATUS_* bit set, and with any bit set."""
    st = np.asarray(status)
    out = {f"chains_{k}": int(np.count_nonzero(st & b)) for k, b in STATUS_BITS.items()}
    out["chains_flagged"] = int(np.count_nonzero(st))
    return out


def max_over_ranks(value, world):
    if world <= 1:
        return float(value)
    from latticeqmc_gb300.distributed import max_over_ranks as mor
    return mor(value)


def time_engine(torch, specs, precision, stab, steps, warmup, stream, seed, dev, world,
                sample_clocks=False, **engine_kw):
    from latticeqmc_gb300 import Engine
    eng = Engine(specs, mode="dqmc", precision=precision, rng="philox", seed=seed,
                 stab_every=stab, device=dev, **engine_kw)
    for _ in range(warmup):
        eng.sweep(1, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    acc0 = [eng.diagnostics(c)["accepted"] for c in range(len(specs))]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev) if sample_clocks else None
    if clocks:
        clocks.start()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    launches = 0
    for _ in range(steps):
        eng.sweep(1, stream=stream.cuda_stream)
        launches += eng.launch_count()
    end.record(stream)
    end.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop() if clocks else None
    ms = max_over_ranks(start.elapsed_time(end) / steps, world)
    if world > 1:
        torch.distributed.barrier()
    diags = [eng.diagnostics(c) for c in range(len(specs))]
    accepted = [(dg["accepted"] - a) / steps for a, dg in zip(acc0, diags)]
    resid = [dg["max_residual"] for dg in diags]
    out = dict(ms=ms, launches=launches, clocks=clk, accepted=accepted,
               resid=max(resid), resid_median=float(np.median(resid)),
               status=status_counts(eng.status()),
               phases={k: float(np.mean([dg["phase_cycles"][k] for dg in diags]))
                       for k in diags[0]["phase_cycles"]},
               subs={k: float(np.mean([dg["sub_cycles"][k] for dg in diags]))
                     for k in diags[0]["sub_cycles"]})
    eng.close()
    return out


def green_difference(specs, stab, dev, precision, sweeps=1, seed=77, **kw):
    """`precision` against fp64 over `sweeps` sweeps from identical fields and uniforms:
    per sweep max|G_precision - G_fp64| over all chains and over the chains whose decisions
    have all agreed so far (the pure precision effect), the number of such chains, and the
    status bits and stabilisation residuals of both engines at the end."""
    from latticeqmc_gb300 import Engine
    rng = np.random.default_rng(seed)
    ref_kw = {k: v for k, v in kw.items() if k == "sweep_order"}
    a = Engine(specs, mode="dqmc", precision="fp64", rng="replay", stab_every=stab, device=dev,
               record=True, **ref_kw)
    b = Engine(specs, mode="dqmc", precision=precision, rng="replay", stab_every=stab, device=dev,
               record=True, **kw)
    total = sum(c.n * c.L for c in specs)
    same = np.ones(len(specs), bool)
    per_sweep, per_sweep_same = [], []
    for _ in range(sweeps):
        u = rng.random(total)
        a.set_uniforms_all(u)
        b.set_uniforms_all(u)
        a.sweep(1)
        b.sweep(1)
        ga, gb = a.green_all(), b.green_all()
        for c in range(len(specs)):
            same[c] &= bool(np.array_equal(a.decisions(c), b.decisions(c)))
        off, dg_same = 0, 0.0
        for c, sp in enumerate(specs):
            k = 2 * sp.n * sp.n
            if same[c]:
                dg_same = max(dg_same, float(np.abs(ga[off:off + k] - gb[off:off + k]).max()))
            off += k
        per_sweep.append(float(np.abs(ga - gb).max()))
        per_sweep_same.append(dg_same if same.any() else None)
    ra = [a.diagnostics(c)["max_residual"] for c in range(len(specs))]
    rb = [b.diagnostics(c)["max_residual"] for c in range(len(specs))]
    out = dict(max_dG=max(per_sweep),
               max_dG_identical_decisions=(max(x for x in per_sweep_same if x is not None)
                                           if same.any() else None),
               max_dG_per_sweep=per_sweep, sweeps_compared=sweeps,
               chains_with_identical_decisions=int(same.sum()), chains=len(specs),
               status_fp64=status_counts(a.status()), status=status_counts(b.status()),
               residual_fp64={"max": max(ra), "median": float(np.median(ra))},
               residual={"max": max(rb), "median": float(np.median(rb))})
    a.close()
    b.close()
    return out


def time_e2e(torch, specs, stab, steps, warmup, stream, dev, world, rank, precision, **kw):
    from latticeqmc_gb300 import Engine
    eng = Engine(specs, mode="dqmc", precision=precision, rng="replay", stab_every=stab, device=dev,
                 **kw)
    total_uni = sum(c.n * c.L for c in specs)
    total_g = sum(2 * c.n * c.n for c in specs)
    steps_all = warmup + steps
    pin_u = torch.empty(steps_all * total_uni, dtype=torch.float64, pin_memory=True)
    pin_u.numpy()[:] = np.random.default_rng(rank).random(steps_all * total_uni)
    pin_g = torch.empty(total_g, dtype=torch.float64, pin_memory=True)
    u_np, g_np = pin_u.numpy(), pin_g.numpy()
    for s in range(warmup):
        eng.set_uniforms_all(u_np[s * total_uni:(s + 1) * total_uni])
        eng.sweep(1, stream=stream.cuda_stream)
        eng.green_all(g_np)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for s in range(warmup, steps_all):
        eng.set_uniforms_all(u_np[s * total_uni:(s + 1) * total_uni])
        eng.sweep(1, stream=stream.cuda_stream)
        eng.green_all(g_np)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / steps, world)
    eng.close()
    return e2e_ms, total_uni * 8, total_g * 8


def batched_vs_sequential(torch, stream, dev, world, rank, steps=2, warmup=1, per_size_seq=4):
    """The 512-chain uneven batch in its launches, against the same chains run one at a
    time (one chain per launch), the latter timed on `per_size_seq` chains of each lattice
    size and scaled to all 512 (the one-chain launch time does not depend on which chain of a
    size it is)."""
    from latticeqmc_gb300 import Engine
    specs, cfg = workload_batched(rank, 128)
    b = time_engine(torch, specs, "fp64", 5, steps, warmup, stream, 4242, dev, world)
    sides = cfg["sides"]
    seq_ms = 0.0
    per_size = {}
    for si, side in enumerate(sides):
        mine = specs[si * 128: si * 128 + per_size_seq]
        t = []
        for sp in mine:
            e = Engine([sp], mode="dqmc", precision="fp64", rng="philox", seed=5, stab_every=5,
                       device=dev)
            e.sweep(1, stream=stream.cuda_stream)
            torch.cuda.synchronize()
            s, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            e.sweep(1, stream=stream.cuda_stream)
            en.record(stream)
            en.synchronize()
            t.append(s.elapsed_time(en))
            e.close()
        per_size[f"{side}x{side}"] = statistics.mean(t)
        seq_ms += statistics.mean(t) * 128
    sites = sum(c.n * c.L for c in specs)
    return {"workload": cfg["workload"], "ms_per_step": b["ms"],
            "value": sites * world / (b["ms"] * 1e-3), "unit": UNIT,
            "sequential_ms_per_sweep": seq_ms, "sequential_value": sites / (seq_ms * 1e-3),
            "speedup_vs_sequential": seq_ms / b["ms"],
            "sequential_ms_per_chain_launch": per_size,
            "sequential_sample": f"{per_size_seq} chains per size, one sweep each after one warm-up, "
                                 "scaled by 128 chains per size",
            "status": b["status"], "steps": steps, "warmup": warmup,
            "gpu_launches": b["launches"]}


def square32(torch, stream, dev, world, rank, steps=1, warmup=1):
    """32x32, beta=6, L=60, fp64e, one chain per SM pair (one wave of the GPU)."""
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    chains = sms // 2
    specs, cfg = workload_square(rank, chains, 32, 6.0, 60, 5, "square32_beta6", "fp64e")
    r = time_engine(torch, specs, "fp64e", 5, steps, warmup, stream, 3232, dev, world,
                    sweep_order="alternate")
    free, _ = torch.cuda.mem_get_info(dev)
    from latticeqmc_gb300 import Engine
    one = Engine(specs[:1], mode="dqmc", precision="fp64e", rng="philox", stab_every=5, device=dev,
                 sweep_order="alternate")
    free1, _ = torch.cuda.mem_get_info(dev)
    one.close()
    per_chain = max(free - free1, 1)
    sites = sum(c.n * c.L for c in specs)
    flops = algorithmic_flops(specs, r["accepted"], 5)
    return {"workload": cfg["workload"], "chains": chains, "stab_every": 5, "sweep_order": "alternate",
            "ms_per_step": r["ms"],
            "value": sites * world / (r["ms"] * 1e-3), "unit": UNIT,
            "sweeps_per_s": 1e3 / r["ms"], "fp64_equivalent_tflops": flops / (r["ms"] * 1e-3) / 1e12,
            "device_bytes_per_chain": per_chain,
            "hbm_admits_chains": int(free // per_chain),
            "note": "timed on one wave (one chain per SM pair); HBM would hold hbm_admits_chains, "
                    "which run in waves of this size at this per-wave time",
            "max_stabilisation_residual": r["resid"], "status": r["status"],
            "steps": steps, "warmup": warmup, "gpu_launches": r["launches"]}


# stabilisation intervals the workload allows: the configuration's 8-16 slices, extended down to
# 6 -- more frequent stabilisation, more work per sweep -- because at 8 the emulated engine's
# G drifts more than 1e-6 between refreshes on a few chains in 16 (the autotuner's residual check)
STAB_RANGE = {"square16_beta8": (6, 16)}


def tuned_settings(args, cfg, precision):
    """Engine settings of the headline engine and the tuning record behind them."""
    from latticeqmc_gb300 import autotune
    default = {"stab_every": cfg["stab_every"], "sweep_order": "alternate"}
    if args.workload == "batched_fp64":
        return {}, None
    rec = autotune.tuned(cfg["sides"][0], cfg["beta"], cfg["L"], precision)
    lo, hi = STAB_RANGE.get(args.workload, (1, 10 ** 6))
    if rec is None:
        return default, {"source": "no autotuner record for this shape: defaults"}
    passing = sorted((r for r in rec["candidates"]
                      if r.get("ok") and lo <= r["stab_every"] <= hi),
                     key=lambda r: r["seconds_per_sweep"])
    if not passing:
        return default, {"source": "no autotuner candidate in the allowed stabilisation range "
                                   "met the accuracy constraint: defaults",
                         "record_chosen": rec["chosen"]}
    kw = {k: v for k, v in autotune.candidate_settings(passing[0]).items()
          if v or k in ("stab_every", "sweep_order", "fp64e_native")}
    keep = ("stab_every", "delay", "oz_stages", "sweep_order", "fp64e_native", "seconds_per_sweep",
            "max_dG", "chains_flagged", "max_residual")
    return kw, {"source": "latticeqmc_gb300/tuning/autotune.json (project autotuner, "
                          f"{rec['chains']} chains, constraint max|dG| <= {rec['tol']} against fp64 "
                          "and no status flag; stab_every restricted to the workload's range "
                          f"{lo}-{hi})",
                "chosen": {k: passing[0].get(k) for k in keep},
                "runner_up": ({k: passing[1].get(k) for k in keep} if len(passing) > 1 else None),
                "candidates_tried": len(rec["candidates"]),
                "candidates_passing": sum(1 for r in rec["candidates"] if r.get("ok"))}


def run_ours(args, rank, world):
    import torch
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    if args.workload == "batched_fp64":
        specs, cfg = workload_batched(rank, args.per_size)
    elif args.workload == "square32_beta6":
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        specs, cfg = workload_square(rank, args.chains or sms // 2, 32, 6.0, 60, 5,
                                     "square32_beta6", "fp64e")
    else:
        specs, cfg = workload_square(rank, args.chains or 64)
    stab = cfg["stab_every"]
    stream = torch.cuda.Stream()
    seed = 12345 + 1000003 * rank
    headline = "fp64" if args.workload == "batched_fp64" else "fp64e"
    # launch settings of the headline engine: the autotuner's choice for this shape when its
    # cache holds one with stab_every in the workload's allowed range, else the defaults
    kw, tuning = tuned_settings(args, cfg, headline)
    old_stab = stab
    stab = kw.pop("stab_every", stab)
    cfg["stab_every"] = stab
    cfg["workload"] = cfg["workload"].replace(f"stab every {old_stab}", f"stab every {stab}")
    cfg["sweep_order"] = kw.get("sweep_order", "down")
    main = time_engine(torch, specs, headline, stab, args.steps, args.warmup, stream, seed, dev,
                       world, sample_clocks=True, **kw)
    order_kw = {"sweep_order": kw["sweep_order"]} if "sweep_order" in kw else {}
    others, subs = {}, {}
    if args.workload == "square16_beta8":
        acc = green_difference(specs, stab, dev, "fp64e", sweeps=args.accuracy_sweeps, **kw)
        main["accuracy"] = acc
        for prec, key in (("fp64", "fp64"), ("mixed", "fp32_mixed")):
            # the other engines on the same workload, stabilisation interval and sweep order
            o = time_engine(torch, specs, prec, stab, args.steps, args.warmup, stream, seed, dev, world,
                            **order_kw)
            od = dict(ms_per_step=o["ms"], status=o["status"],
                      max_stabilisation_residual=o["resid"])
            if prec != "fp64":
                od.update(green_difference(specs, stab, dev, prec, sweeps=1, **order_kw))
            others[key] = od
        if not args.no_subrecords:
            subs["batched_fp64"] = batched_vs_sequential(torch, stream, dev, world, rank)
            subs["square32_beta6"] = square32(torch, stream, dev, world, rank)
    e2e_ms, h2d, d2h = time_e2e(torch, specs, stab, args.steps, args.warmup, stream, dev, world,
                                rank, headline, **kw)
    peak = fp64_peak_tflops(torch) if rank == 0 else None
    return dict(ms=main["ms"], sites=sum(c.n * c.L for c in specs), chains=len(specs),
                flops=algorithmic_flops(specs, main["accepted"], stab), launches=main["launches"],
                clocks=main["clocks"], e2e_ms=e2e_ms, h2d=h2d, d2h=d2h, cfg=cfg,
                resid=main["resid"], resid_median=main["resid_median"], status=main["status"],
                peak=peak, specs=specs, phases=main["phases"], subs_cycles=main["subs"],
                others=others, subrecords=subs, headline=headline,
                accuracy=main.get("accuracy"), tuning=tuning)


def roofline(r, args):
    fp64_eq = r["flops"] / (r["ms"] * 1e-3) / 1e12
    if r["headline"] == "fp64e":
        peaks = {}
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                peaks = json.load(f)
        except (OSError, ValueError):
            pass
        tpeak = peaks.get("bf16_tflops_sustained")
        tsrc = "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)"
        if tpeak is None:
            tpeak, tsrc = 1700.0, "fallback sustained bf16 figure (of fallback)"
        achieved = 36.0 * fp64_eq
        full = args.workload == "square16_beta8" and (args.chains or 64) == 64
        roof = {"bound": "tensor", "achieved": achieved, "peak": tpeak, "unit": "TFLOP/s",
                "frac": achieved / tpeak, "peak_source": tsrc,
                "traffic": FP64E_TRAFFIC if full else None,
                "traffic_unit": "DRAM bytes per launch (one sweep of all chains)",
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the "
                                  "fp64e sweep kernel on this workload (mean of 2 launches)",
                "kernel": "sweep kernel of the fp64e engine (BF16 slice products: 36 per "
                          "algorithmic float64 flop)",
                "fp64_equivalent": {"achieved": fp64_eq, "peak": r["peak"], "unit": "TFLOP/s",
                                    "frac": fp64_eq / r["peak"] if r["peak"] else None,
                                    "peak_source": "cuBLAS DGEMM 4096^3 measured in this run"}}
        dtype = "f64 (GEMMs emulated: 8 BF16 slices, FP32 tensor-core accumulation)"
    else:
        roof = {"bound": "fp64", "achieved": fp64_eq, "peak": r["peak"], "unit": "TFLOP/s",
                "frac": fp64_eq / r["peak"] if r["peak"] else None, "traffic": None,
                "peak_source": "cuBLAS DGEMM 4096^3 measured in this run "
                               "(MEASURED_PEAKS.json carries no float64 figure)",
                "kernel": "sweep kernel of the float64 engine (all launch buckets of one sweep)"}
        dtype = "f64"
    return roof, dtype


def make_line(args, r, world, cpu):
    """The JSON line rank 0 prints from its (max-over-ranks) measurements."""
    sites_all = r["sites"] * world
    value = sites_all / (r["ms"] * 1e-3)
    e2e = sites_all / (r["e2e_ms"] * 1e-3)
    roof, dtype = roofline(r, args)
    tot = max(sum(r["phases"].values()), 1.0)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms"],
        "sweeps_per_s": 1e3 / r["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtype, "data": "synthetic",
        "config": dict(r["cfg"], **config_extras(world)),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"], "ms_per_step": r["e2e_ms"]},
        "gpu_launches": r["launches"],
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": r["clocks"],
        "status": dict(r["status"], max_stabilisation_residual=r["resid"],
                       median_stabilisation_residual=r["resid_median"]),
        "phase_share": {k: v / tot for k, v in r["phases"].items()},
        "sub_share": {k: v / tot for k, v in r["subs_cycles"].items()},
        "tuning": r.get("tuning"),
    }
    if r.get("accuracy"):
        acc = dict(r["accuracy"])
        acc["meets_max_dG_1e-6"] = bool(acc["max_dG"] <= 1e-6)
        line["accuracy"] = acc
    for key, od in r["others"].items():
        entry = dict(od, value=sites_all / (od["ms_per_step"] * 1e-3), unit=UNIT)
        if key == "fp64":
            entry["speedup_of_value"] = od["ms_per_step"] / r["ms"]
        else:
            entry["speedup_vs_fp64"] = r["others"]["fp64"]["ms_per_step"] / od["ms_per_step"]
            entry["meets_max_dG_1e-6"] = bool(od["max_dG"] <= 1e-6)
        line[key] = entry
    line.update(r["subrecords"])
    return line


def reference_arm(args):
    """The reference's CPU path (the port) on the host cores: each step is one bounded
    sample of every lattice size on every core; `value` is the per-site rate of the samples
    applied to one sweep of the workload, `ms_per_step` the wall time of a step."""
    if args.workload == "batched_fp64":
        specs, cfg = workload_batched(0, args.per_size)
    elif args.workload == "square32_beta6":
        specs, cfg = workload_square(0, args.chains or 76, 32, 6.0, 60, 5, "square32_beta6", "fp64e")
    else:
        specs, cfg = workload_square(0, args.chains or 64)
    vals, walls = [], []
    last = None
    for s in range(args.warmup + args.steps):
        last = cpu_baseline(specs, cfg, seconds_per_size=min(args.cpu_seconds, 1.0))
        if s >= args.warmup:
            vals.append(last["value"])
            walls.append(last["wall_seconds"])
    v = statistics.mean(vals)
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.mean(walls) * 1e3,
            "step": "one bounded sample of the reference's sweep on every host core (the rate "
                    "is the slope between two sample lengths, applied to one sweep of all chains)",
            "sweep_seconds_extrapolated": sum(c.n * c.L for c in specs) / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": dict(cfg, **config_extras(1)),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": last["cores"],
                             "kind": "port", "sample": last["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def launcher_command(argv, gpus, port=None):
    """torch.distributed.run command that starts `gpus` ranks of this script on 127.0.0.1."""
    if port is None:
        with socket.socket() as s:
            s.bind(("127.0.0.1", 0))
            port = s.getsockname()[1]
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
            f"--nproc-per-node={gpus}", "--master-addr", "127.0.0.1", f"--master-port={port}",
            os.path.abspath(__file__), *argv]


def check_world(gpus, env):
    """World size of this process: `gpus` must match the launcher's WORLD_SIZE if one is
    set.  Returns None when bench.py has to start the ranks itself."""
    if "WORLD_SIZE" not in env:
        return None if gpus > 1 else 1
    world = int(env["WORLD_SIZE"])
    if world != gpus:
        raise SystemExit(f"bench.py: --gpus {gpus} but the launcher started {world} ranks")
    return world


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="square16_beta8",
                    choices=["square16_beta8", "batched_fp64", "square32_beta6"])
    ap.add_argument("--chains", type=int, default=0,
                    help="chains of the square workloads (0: 64 at 16x16, one wave at 32x32)")
    ap.add_argument("--accuracy-sweeps", type=int, default=10,
                    help="sweeps of the fp64e-vs-fp64 comparison from identical inputs")
    ap.add_argument("--cpu-seconds", type=float, default=2.5,
                    help="seconds of CPU sampling per lattice size and process")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-subrecords", action="store_true",
                    help="leave out the batched_fp64 and square32_beta6 sub-records")
    ap.add_argument("--per-size", type=int, default=128,
                    help="chains per lattice size (128 is the workload; smaller for profiling)")
    return ap.parse_args(argv)


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    args = parse(argv)
    world = check_world(args.gpus, os.environ)
    if world is None:
        return subprocess.call(launcher_command(argv, args.gpus))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(reference_arm(args)))
        return 0
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    r = run_ours(args, rank, world)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(r["specs"], r["cfg"], seconds_per_size=args.cpu_seconds)
        one = cpu_baseline(r["specs"], r["cfg"], seconds_per_size=args.cpu_seconds, cores=1)
        for d in (cpu, one):
            d.pop("sweep_seconds", None)
            d.pop("wall_seconds", None)
        cpu["single_process"] = {k: one[k] for k in ("value", "unit", "cores", "sample")}
    if rank == 0:
        print(json.dumps(make_line(args, r, world, cpu)))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
