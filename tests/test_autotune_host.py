"""The autotuner's search space and its accuracy-constrained choice, with stand-ins for the
timing and the float64 comparison (no GPU)."""
import json

from latticeqmc_gb300 import autotune as at


def test_candidates_cover_the_search_space_without_duplicates():
    c = at.default_candidates("fp64e")
    keys = [json.dumps(x, sort_keys=True) for x in c]
    assert len(keys) == len(set(keys)) == 5 * 2 * len(at.NATIVE_SETS)
    assert {x["sweep_order"] for x in c} == {"down", "alternate"}
    assert {x["stab_every"] for x in c} == {6, 8, 10, 12, 16}
    assert {tuple(x["fp64e_native"]) for x in c} == set(at.NATIVE_SETS)
    assert all(x["delay"] == 0 and x["oz_stages"] == 0 for x in c)
    assert all("fp64e_native" not in x for x in at.default_candidates("fp64"))
    best = dict(c[3])
    r = at.refine_candidates(best, "fp64e")
    assert {x["delay"] for x in r} == {0, 8, 16, 32, 48}
    assert {x["oz_stages"] for x in r} == {0, 1, 2, 3}
    assert all(x["stab_every"] == best["stab_every"] and x["fp64e_native"] == best["fp64e_native"] for x in r)
    assert {x["oz_stages"] for x in at.refine_candidates(best, "fp64")} == {0}


def test_second_pass_refines_around_the_fastest_passing_grid_point(monkeypatch, tmp_path):
    monkeypatch.setattr(at, "_specs", lambda *a: [])
    monkeypatch.setattr(at, "time_candidate",
                        lambda specs, p, c, s, d=0: (1.0 if c["stab_every"] != 8 else 0.5)
                        - 0.01 * (c["delay"] == 32) - 0.001 * len(c.get("fp64e_native", [])))
    monkeypatch.setattr(at, "check_candidate",
                        lambda specs, p, c, s, d=0, ref_cache=None: {
                            "max_dG": 1e-8, "chains_diverged": 0, "max_residual": 0.0,
                            "fp64_chains_flagged": 0,
                            "chains_flagged": 0 if "lu" in c.get("fp64e_native", []) else 1})
    rec = at.autotune(16, 8.0, 80, "fp64e", cache=str(tmp_path / "t.json"), log=None)
    ch = rec["chosen"]
    assert ch["stab_every"] == 8 and ch["delay"] == 32 and ch["fp64e_native"] == ["lu", "lu_rhs"]
    kw = at.settings(rec)
    assert kw["fp64e_native"] == ("lu", "lu_rhs") and kw["delay"] == 32


def test_fastest_setting_meeting_the_bar_is_chosen_and_cached(tmp_path, monkeypatch):
    speed = {6: 0.6, 8: 0.5, 10: 0.45, 12: 0.40, 16: 0.35}
    monkeypatch.setattr(at, "_specs", lambda *a: [])
    monkeypatch.setattr(at, "time_candidate",
                        lambda specs, p, c, s, d=0: speed[c["stab_every"]] * (0.8 if c["sweep_order"] == "alternate" else 1))

    def check(specs, p, c, s, d=0, ref_cache=None):
        # stab >= 12 drifts; stab 10 passes max|dG| but one chain is flagged
        return {"max_dG": 1e-7 if c["stab_every"] < 12 else 3e-6,
                "chains_diverged": 0, "chains_flagged": 1 if c["stab_every"] == 10 else 0,
                "max_residual": 0.0, "fp64_chains_flagged": 0}
    monkeypatch.setattr(at, "check_candidate", check)
    cands = [{"stab_every": s, "delay": 0, "sweep_order": o, "oz_stages": 0}
             for s in speed for o in ("down", "alternate")]
    cache = tmp_path / "t.json"
    rec = at.autotune(16, 8.0, 80, "fp64e", candidates=cands, cache=str(cache), log=None)
    assert rec["chosen"]["stab_every"] == 8 and rec["chosen"]["sweep_order"] == "alternate"
    assert rec["runner_up"]["stab_every"] == 6 and rec["runner_up"]["sweep_order"] == "alternate"
    assert at.tuned(16, 8.0, 80, "fp64e", cache=str(cache))["chosen"] == rec["chosen"]
    assert at.settings(rec) == {"stab_every": 8, "delay": 0, "sweep_order": "alternate", "oz_stages": 0}
    assert rec["candidates"] and len(rec["candidates"]) == len(cands)   # given candidates: one pass
    assert json.loads(cache.read_text())["square16_beta8_L80_fp64e"]["shape"] == rec["shape"]
