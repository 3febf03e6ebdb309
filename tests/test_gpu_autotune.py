"""The autotuner on the GPU: a small search on a 4x4 lattice times and checks each candidate
against the float64 engine, and writes a record the bench can read back."""
import json

import pytest

from latticeqmc_gb300 import autotune as at

pytestmark = pytest.mark.gpu


def test_small_search_times_checks_and_caches(tmp_path):
    cands = [{"stab_every": 5, "delay": 0, "sweep_order": "down", "oz_stages": 0, "fp64e_native": []},
             {"stab_every": 5, "delay": 8, "sweep_order": "alternate", "oz_stages": 2,
              "fp64e_native": ["lu", "lu_rhs"]}]
    cache = tmp_path / "t.json"
    rec = at.autotune(4, 2.0, 20, "fp64e", candidates=cands, chains=2, time_chains=4, time_sweeps=1,
                      acc_sweeps=2, cache=str(cache), log=print)
    assert len(rec["candidates"]) == 2
    for row in rec["candidates"]:
        assert row["seconds_per_sweep"] > 0
        assert row["max_dG"] < 1e-8 and row["chains_diverged"] == 0
        assert row["ok"]
    assert rec["chosen"] is not None and rec["runner_up"] is not None
    kw = at.settings(rec)
    assert set(kw) == {"stab_every", "delay", "sweep_order", "oz_stages", "fp64e_native"}
    assert json.loads(cache.read_text())["square4_beta2_L20_fp64e"]["chosen"] == rec["chosen"]
