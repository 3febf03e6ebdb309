"""Accuracy-constrained autotuner of the sweep engine's launch parameters.

For one workload shape (square lattice side, beta, L, precision) it times candidate settings of

    stab_every    slices between stabilised refreshes of G
    sweep_order   'down' (the reference's order) or 'alternate'
    fp64e_native  (fp64e) product categories kept in native float64
    delay         depth k of the delayed rank-k updates (0: the engine's rule)
    oz_stages     stage buffers of the emulated GEMM's copy / MMA ring (fp64e; 0: the rule)

on the workload's chain count, checks each against the float64 engine run from identical
fields and uniforms with the same stab_every and sweep order (the same chains by default),
and picks the fastest setting that meets

    max|G - G_fp64| <= tol after every compared sweep, identical accept/reject decisions, and
    no chain raising a status bit (LQMC_STATUS_DRIFT: a stabilisation residual above 1e-6).

The search is two coordinate passes: a grid over the settings that decide accuracy
(stab_every x sweep order x native categories) at the default delay and stage count, then
every delay and stage count around the fastest passing grid point.

Results go to a JSON cache keyed by the workload shape (``tuning/autotune.json`` beside this
module); ``tuned(...)`` reads a record back.  Without a record the engine's own rules apply
(engine.auto_stab_every, the delay and stage rule of the C layer).

    python -m latticeqmc_gb300.autotune --side 16 --beta 8 --L 80 --precision fp64e
"""
import json
import os
import time

import numpy as np

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning", "autotune.json")


def shape_key(side, beta, L, precision):
    return f"square{side}_beta{beta:g}_L{L}_{precision}"


def _specs(side, beta, L, chains, seed):
    from .engine import ChainSpec
    from .hubbard import HubbardModel
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(side)
    K = m.ham_kinetic()
    n = side * side
    rng = np.random.default_rng(seed)
    return [ChainSpec(K, 4.0, beta, L, (2 * rng.integers(0, 2, (n, L)) - 1).astype(np.int8))
            for _ in range(chains)]


def _engine(specs, precision, cand, device, rng, record=False):
    from .engine import Engine
    kw = {}
    if precision == "fp64e" and "fp64e_native" in cand:
        kw["fp64e_native"] = tuple(cand["fp64e_native"])
    return Engine(specs, mode="dqmc", precision=precision, rng=rng, seed=1, record=record,
                  stab_every=cand["stab_every"], delay=cand.get("delay", 0), device=device,
                  sweep_order=cand["sweep_order"], oz_stages=cand.get("oz_stages", 0), **kw)


def time_candidate(specs, precision, cand, sweeps, device=0):
    """Seconds per sweep of `cand` (Philox uniforms, CUDA events, after two warm-up sweeps:
    the alternating order's first sweep builds its stacks from scratch)."""
    import torch
    eng = _engine(specs, precision, cand, device, "philox")
    try:
        eng.sweep(2)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        eng.sweep(sweeps)
        e.record()
        e.synchronize()
        return s.elapsed_time(e) * 1e-3 / sweeps
    finally:
        eng.close()


def check_candidate(specs, precision, cand, sweeps, device=0, ref_cache=None):
    """Worst max|G - G_fp64| over `sweeps` sweeps from identical inputs, the chains whose
    decisions differed, and the status bits of both engines."""
    ref_cache = {} if ref_cache is None else ref_cache
    key = (cand["stab_every"], cand["sweep_order"])
    rng = np.random.default_rng(97)
    total = sum(c.n * c.L for c in specs)
    us = [rng.random(total) for _ in range(sweeps)]
    if key not in ref_cache:
        ref = _engine(specs, "fp64", {"stab_every": cand["stab_every"],
                                      "sweep_order": cand["sweep_order"]}, device, "replay", True)
        gs, decs = [], []
        try:
            for u in us:
                ref.set_uniforms_all(u)
                ref.sweep(1)
                gs.append(ref.green_all())
                decs.append([ref.decisions(c).copy() for c in range(len(specs))])
            st = ref.status()
        finally:
            ref.close()
        ref_cache[key] = (gs, decs, st)
    gs, decs, st_ref = ref_cache[key]
    eng = _engine(specs, precision, cand, device, "replay", True)
    worst, diverged = 0.0, set()
    try:
        for k, u in enumerate(us):
            eng.set_uniforms_all(u)
            eng.sweep(1)
            worst = max(worst, float(np.abs(eng.green_all() - gs[k]).max()))
            for c in range(len(specs)):
                if not np.array_equal(eng.decisions(c), decs[k][c]):
                    diverged.add(c)
        st = eng.status()
        resid = max(eng.diagnostics(c)["max_residual"] for c in range(len(specs)))
    finally:
        eng.close()
    return {"max_dG": worst, "chains_diverged": len(diverged),
            "chains_flagged": int(np.count_nonzero(st)), "max_residual": resid,
            "fp64_chains_flagged": int(np.count_nonzero(st_ref))}


# native-float64 category sets tried for fp64e: all emulated, and the stabilised inverse's LU
# (with or without its right-hand side) native.  Keeping the QR updates and B-chain products
# native as well halves the speed without bringing every chain's residual below 1e-6 at
# stab_every 8, so it is not searched.
NATIVE_SETS = ((), ("lu",), ("lu", "lu_rhs"))


def _dedup(cands):
    seen, out = set(), []
    for c in cands:
        k = json.dumps(c, sort_keys=True)
        if k not in seen:
            seen.add(k)
            out.append(c)
    return out


def default_candidates(precision, stabs=(6, 8, 10, 12, 16), orders=("down", "alternate"),
                       natives=NATIVE_SETS):
    """The first pass: every stab_every x sweep order (x fp64e native set) at the engine's
    default delay and stage count."""
    nats = natives if precision == "fp64e" else (None,)
    cands = []
    for order in orders:
        for nat in nats:
            for st in stabs:
                c = {"stab_every": st, "delay": 0, "sweep_order": order, "oz_stages": 0}
                if nat is not None:
                    c["fp64e_native"] = list(nat)
                cands.append(c)
    return _dedup(cands)


def refine_candidates(best, precision, delays=(8, 16, 32, 48), stages=(1, 2, 3)):
    """The second pass: each delay and (fp64e) each stage count around `best`."""
    cands = [dict(best, delay=k) for k in delays]
    if precision == "fp64e":
        cands += [dict(best, oz_stages=sg) for sg in stages]
    keys = ("stab_every", "delay", "sweep_order", "oz_stages", "fp64e_native")
    return _dedup([{k: c[k] for k in keys if k in c} for c in cands])


def _run(cands, specs_time, specs_acc, precision, time_sweeps, acc_sweeps, tol, device, ref_cache,
         label, log):
    rows = []
    for cand in cands:
        t0 = time.perf_counter()
        try:
            sec = time_candidate(specs_time, precision, cand, time_sweeps, device)
            acc = check_candidate(specs_acc, precision, cand, acc_sweeps, device, ref_cache)
            ok = acc["max_dG"] <= tol and acc["chains_flagged"] == 0 and acc["chains_diverged"] == 0
            row = dict(cand, seconds_per_sweep=sec, ok=ok, **acc)
        except RuntimeError as e:            # a setting the engine refuses (shared memory)
            row = dict(cand, ok=False, error=str(e))
        rows.append(row)
        if log:
            log(f"autotune {label} {cand}: "
                + (f"{row['seconds_per_sweep'] * 1e3:.1f} ms/sweep, max|dG| {row['max_dG']:.1e}, "
                   f"flagged {row['chains_flagged']}, diverged {row['chains_diverged']}, "
                   f"{'ok' if row['ok'] else 'rejected'}"
                   if "error" not in row else f"refused: {row['error']}")
                + f" [{time.perf_counter() - t0:.0f}s]")
    return rows


def autotune(side, beta, L, precision="fp64e", candidates=None, chains=64, time_chains=64,
             time_sweeps=2, acc_sweeps=4, tol=1e-6, device=0, cache=CACHE, log=print):
    """Time and check the candidates (given, or the two passes above); cache and return the
    record of the workload shape."""
    label = shape_key(side, beta, L, precision)
    specs_acc = _specs(side, beta, L, chains, 4321)
    specs_time = specs_acc if time_chains == chains else _specs(side, beta, L, time_chains, 4321)
    ref_cache = {}
    args = (specs_time, specs_acc, precision, time_sweeps, acc_sweeps, tol, device, ref_cache, label, log)
    if candidates is not None:
        rows = _run(candidates, *args)
    else:
        rows = _run(default_candidates(precision), *args)
        passing = sorted((r for r in rows if r["ok"]), key=lambda r: r["seconds_per_sweep"])
        if passing:
            best = {k: v for k, v in passing[0].items()
                    if k in ("stab_every", "delay", "sweep_order", "oz_stages", "fp64e_native")}
            done = {json.dumps({k: r[k] for k in best if k in r}, sort_keys=True) for r in rows}
            extra = [c for c in refine_candidates(best, precision)
                     if json.dumps(c, sort_keys=True) not in done]
            rows += _run(extra, *args)
    passing = sorted((r for r in rows if r["ok"]), key=lambda r: r["seconds_per_sweep"])
    record = {"shape": label, "chains": chains, "time_chains": time_chains, "tol": tol,
              "time_sweeps": time_sweeps, "acc_sweeps": acc_sweeps,
              "chosen": passing[0] if passing else None,
              "runner_up": passing[1] if len(passing) > 1 else None, "candidates": rows}
    if cache:
        os.makedirs(os.path.dirname(cache), exist_ok=True)
        data = {}
        if os.path.exists(cache):
            with open(cache) as f:
                data = json.load(f)
        data[record["shape"]] = record
        with open(cache, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
    return record


def tuned(side, beta, L, precision, cache=CACHE):
    """The cached record of a workload shape, or None."""
    try:
        with open(cache) as f:
            return json.load(f).get(shape_key(side, beta, L, precision))
    except (OSError, ValueError):
        return None


def settings(record):
    """Engine keyword arguments of a record's chosen setting."""
    return candidate_settings(record["chosen"])


def candidate_settings(c):
    """Engine keyword arguments of one candidate row."""
    kw = {"stab_every": c["stab_every"], "delay": c["delay"], "sweep_order": c["sweep_order"],
          "oz_stages": c["oz_stages"]}
    if "fp64e_native" in c:
        kw["fp64e_native"] = tuple(c["fp64e_native"])
    return kw


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description="accuracy-constrained autotuner of the sweep engine")
    ap.add_argument("--side", type=int, default=16)
    ap.add_argument("--beta", type=float, default=8.0)
    ap.add_argument("--L", type=int, default=80)
    ap.add_argument("--precision", default="fp64e")
    ap.add_argument("--chains", type=int, default=64, help="chains of the accuracy check")
    ap.add_argument("--time-chains", type=int, default=64, help="chains of the timing")
    a = ap.parse_args()
    rec = autotune(a.side, a.beta, a.L, a.precision, chains=a.chains, time_chains=a.time_chains)
    print(json.dumps({k: rec[k] for k in ("shape", "chosen", "runner_up")}, indent=1))
