"""bench.py's host logic without a GPU: the --gpus launcher, the world-size check, and the
JSON line two ranks produce (max step time over ranks, whole-job value), over gloo."""
import json
import os
import socket

import numpy as np
import pytest

import bench


def test_world_size_check():
    assert bench.check_world(1, {}) == 1
    assert bench.check_world(4, {}) is None            # bench.py starts the ranks itself
    assert bench.check_world(2, {"WORLD_SIZE": "2"}) == 2
    with pytest.raises(SystemExit):
        bench.check_world(8, {"WORLD_SIZE": "1"})


def test_launcher_command_starts_n_local_ranks():
    cmd = bench.launcher_command(["--gpus", "4", "--steps", "2"], 4, port=29555)
    assert cmd[1:3] == ["-m", "torch.distributed.run"]
    assert "--nproc-per-node=4" in cmd and "--master-port=29555" in cmd
    assert cmd[cmd.index("--master-addr") + 1] == "127.0.0.1"
    assert cmd[-4:] == ["--gpus", "4", "--steps", "2"]
    assert os.path.samefile(cmd[-5], os.path.join(bench.ROOT, "bench.py"))


def test_main_without_launcher_relaunches(monkeypatch):
    seen = {}
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.setattr(bench.subprocess, "call", lambda cmd: seen.setdefault("cmd", cmd) and 0)
    assert bench.main(["--gpus", "2", "--steps", "1"]) == 0
    assert "--nproc-per-node=2" in seen["cmd"]


def _stand_in_result(ms, world):
    """What run_ours returns, for a stand-in engine whose step takes `ms` on this rank."""
    class Spec:
        n, L = 256, 80
    specs = [Spec()] * 4
    cfg = {"workload": "stand-in", "chains": 4, "sides": [16], "beta": 8.0, "L": 80,
           "stab_every": 8}
    return dict(ms=bench.max_over_ranks(ms, world), sites=4 * 256 * 80, chains=4,
                flops=bench.algorithmic_flops(specs, [100.0] * 4, 8), launches=1,
                clocks=None, e2e_ms=bench.max_over_ranks(ms + 1.0, world), h2d=8, d2h=16,
                cfg=cfg, resid=1e-9, resid_median=1e-10, status=bench.status_counts([0, 4, 0, 0]),
                peak=1.0, specs=specs, phases={"update": 1.0}, subs_cycles={"lu": 0.5},
                others={}, subrecords={}, headline="fp64e", accuracy=None)


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        args = bench.parse(["--gpus", str(world), "--steps", "3"])
        r = _stand_in_result(10.0 + 5.0 * rank, world)
        if rank == 0:
            with open(out, "w") as f:
                f.write(json.dumps(bench.make_line(args, r, world, None)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_rank():
    import torch.multiprocessing as tmp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = os.path.join(os.path.dirname(__file__), "..", ".pytest_cache", "bench_line.json")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    tmp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    line = json.loads(open(out).read())
    assert line["n_gpus"] == 2 and line["scaling"] == "weak"
    assert line["ms_per_step"] == 15.0                      # the slower rank
    assert np.isclose(line["value"], 2 * 4 * 256 * 80 / 15e-3)
    assert np.isclose(line["e2e"]["value"], 2 * 4 * 256 * 80 / 16e-3)
    assert line["status"]["chains_drift"] == 1 and line["status"]["chains_flagged"] == 1
    assert line["config"]["parallelism"] == "chains sharded over 2 GPU(s)"


def test_status_counts_every_bit():
    c = bench.status_counts(np.array([0, 1, 2, 4, 8, 12]))
    assert c == {"chains_nonfinite": 1, "chains_singular": 1, "chains_drift": 2,
                 "chains_timeout": 2, "chains_flagged": 5}


def test_tuned_settings_take_the_fastest_passing_candidate_in_the_workloads_range(monkeypatch):
    """bench.tuned_settings: candidates outside the workload's stab_every range are skipped,
    every tuned setting (native categories included) reaches the engine, and the record's
    chosen and runner-up are reported."""
    import argparse
    from latticeqmc_gb300 import autotune

    def row(stab, sec, ok, **kw):
        return dict({"stab_every": stab, "delay": 0, "sweep_order": "alternate", "oz_stages": 0,
                     "fp64e_native": [], "seconds_per_sweep": sec, "ok": ok, "max_dG": 1e-9,
                     "chains_flagged": 0 if ok else 1, "max_residual": 1e-7}, **kw)
    rec = {"chains": 64, "tol": 1e-6, "chosen": None,
           "candidates": [row(4, 0.30, True), row(6, 0.47, True, delay=48),
                          row(6, 0.48, True, fp64e_native=["lu"]), row(8, 0.42, False),
                          row(20, 0.35, True)]}
    monkeypatch.setattr(autotune, "tuned", lambda *a: rec)
    args = argparse.Namespace(workload="square16_beta8")
    cfg = {"sides": [16], "beta": 8.0, "L": 80, "stab_every": 8}
    kw, info = bench.tuned_settings(args, cfg, "fp64e")
    assert kw == {"stab_every": 6, "delay": 48, "sweep_order": "alternate", "fp64e_native": ()}
    assert info["chosen"]["seconds_per_sweep"] == 0.47
    assert info["runner_up"]["fp64e_native"] == ["lu"]
    assert info["candidates_passing"] == 4
    monkeypatch.setattr(autotune, "tuned", lambda *a: None)
    kw, info = bench.tuned_settings(args, cfg, "fp64e")
    assert kw == {"stab_every": 8, "sweep_order": "alternate"} and "defaults" in info["source"]
