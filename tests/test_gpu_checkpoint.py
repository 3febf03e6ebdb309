"""Checkpoint / resume of chains and of batched (U, beta) scans: an interrupted run that
resumes from its checkpoint ends with exactly the numbers of an uninterrupted run."""
import numpy as np
import pytest

from latticeqmc_gb300 import ChainSpec, Engine, HubbardModel, scan

pytestmark = pytest.mark.gpu


def _specs(seed=5):
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(4)
    K = m.ham_kinetic()
    rng = np.random.default_rng(seed)
    return K, [ChainSpec(K, u, 2.0, 20, (2 * rng.integers(0, 2, (16, 20)) - 1).astype(np.int8))
               for u in (2.0, 4.0, 6.0)]


@pytest.mark.parametrize("precision", ["fp64", "fp64e"])
def test_engine_checkpoint_resume_is_bit_identical(tmp_path, precision):
    K, specs = _specs()
    kw = dict(mode="dqmc", precision=precision, rng="philox", seed=11, stab_every=5)
    straight = Engine(specs, **kw)
    straight.sweep(3)
    straight.reset_measurements()
    straight.sweep(4, measure=True)
    ref = [(straight.field(c), straight.green_sum(c)[0], straight.observables_raw(c))
           for c in range(len(specs))]
    straight.close()

    first = Engine(specs, **kw)
    first.sweep(3)
    first.reset_measurements()
    first.sweep(2, measure=True)
    path = tmp_path / "ck.npz"
    first.checkpoint(path)
    first.close()
    second = Engine(specs, **kw)
    second.restore(path)
    assert second.diagnostics(0)["sweeps"] == 5
    second.sweep(2, measure=True)
    for c in range(len(specs)):
        f, g, o = ref[c]
        assert np.array_equal(second.field(c), f)
        assert np.array_equal(second.green_sum(c)[0], g)
        assert np.array_equal(second.observables_raw(c), o)
    second.close()


def test_restore_rejects_other_chains(tmp_path):
    K, specs = _specs()
    eng = Engine(specs, mode="dqmc", rng="philox", seed=1, stab_every=5)
    eng.sweep(1)
    path = tmp_path / "ck.npz"
    eng.checkpoint(path)
    eng.close()
    other = Engine(specs[:2], mode="dqmc", rng="philox", seed=1, stab_every=5)
    with pytest.raises(ValueError):
        other.restore(path)
    other.close()


def test_interrupted_scan_resumes_to_the_same_result(tmp_path):
    K, _ = _specs()
    points = [(2.0, 1.0), (4.0, 1.0), (4.0, 2.0)]
    kw = dict(time_steps=20, warmup=4, sweeps=6, chains_per_point=2, seed=3, stab_every=5)
    full = scan(K, points, **kw)
    path = str(tmp_path / "scan.npz")
    assert scan(K, points, checkpoint=path, checkpoint_every=3, stop_after=5, **kw) is None
    resumed = scan(K, points, checkpoint=path, checkpoint_every=3, **kw)
    assert np.array_equal(resumed["green"], full["green"])
    assert np.array_equal(resumed["count"], full["count"])
    assert list(resumed["count"]) == [12, 12, 12]
    for k in ("kinetic_energy", "potential_energy", "double_occupancy", "density"):
        assert np.array_equal(resumed[k], full[k])
    # half filling at mu = 0
    assert np.allclose(full["density"], 1.0, atol=0.1)
