"""The control flow of batched scans (checkpoint cadence, warm-up / measurement split,
resume) on the CPU, with a deterministic stand-in for the GPU engine."""
import os

import numpy as np
import pytest

import latticeqmc_gb300.scans as scan_mod


class FakeEngine:
    """Counts sweeps; a measured sweep adds (sweep index + 1) to every sum of every chain."""

    def __init__(self, specs, rng, seed, **kw):
        self.n = len(specs)
        self.sites = specs[0].n
        self.done = 0
        self.gsum = np.zeros(self.n)
        self.count = np.zeros(self.n, dtype=np.int64)
        self.sweep_log = []

    def restore(self, path):
        z = np.load(path)
        self.done, self.gsum, self.count = int(z["done"]), z["gsum"].copy(), z["count"].copy()

    def checkpoint(self, path):
        np.savez(path, done=self.done, gsum=self.gsum, count=self.count)

    def diagnostics(self, c):
        return {"sweeps": self.done}

    def reset_measurements(self):
        self.gsum[:] = 0.0
        self.count[:] = 0

    def sweep(self, n, measure=False):
        self.sweep_log.append((n, measure))
        for _ in range(n):
            self.done += 1
            if measure:
                self.gsum += self.done
                self.count += 1

    def green_sum(self, c):
        return np.full((2, self.sites, self.sites), self.gsum[c]), int(self.count[c])

    def observables_raw(self, c):
        return np.array([self.count[c], self.gsum[c], 2 * self.gsum[c], 3 * self.gsum[c], self.count[c]],
                        dtype=np.float64)

    def close(self):
        pass


@pytest.fixture
def fake(monkeypatch):
    engines = []

    def make(*a, **k):
        e = FakeEngine(*a, **k)
        engines.append(e)
        return e
    monkeypatch.setattr(scan_mod, "Engine", make)
    return engines


def test_scan_splits_warmup_and_measurement(fake):
    K = -np.eye(4, k=1) - np.eye(4, k=-1)
    out = scan_mod.scan(K, [(2.0, 1.0), (4.0, 1.0)], time_steps=10, warmup=3, sweeps=5,
                        chains_per_point=2)
    assert list(out["count"]) == [10, 10]
    # measured sweeps are 4..8: sum 30 per chain, 2 chains per point, mean 30 / 5 = 6
    np.testing.assert_allclose(out["green"], 6.0)
    np.testing.assert_allclose(out["density"], 1.0)
    assert fake[0].sweep_log == [(3, False), (5, True)]


def test_interrupted_scan_resumes_to_the_same_numbers(fake, tmp_path):
    K = -np.eye(4, k=1) - np.eye(4, k=-1)
    pts = [(2.0, 1.0), (4.0, 2.0)]
    full = scan_mod.scan(K, pts, time_steps=10, warmup=4, sweeps=7)
    ck = str(tmp_path / "scan.npz")
    assert scan_mod.scan(K, pts, time_steps=10, warmup=4, sweeps=7, checkpoint=ck,
                         checkpoint_every=3, stop_after=5) is None
    assert os.path.isfile(ck)
    first = fake[-1]
    assert first.done == 5 and all(n <= 3 for n, _ in first.sweep_log)
    resumed = scan_mod.scan(K, pts, time_steps=10, warmup=4, sweeps=7, checkpoint=ck,
                            checkpoint_every=3)
    assert fake[-1].done == 11
    np.testing.assert_array_equal(resumed["green"], full["green"])
    np.testing.assert_array_equal(resumed["count"], full["count"])
    for k in ("kinetic_energy", "potential_energy", "double_occupancy", "density"):
        np.testing.assert_array_equal(resumed[k], full[k])
    assert not os.path.isfile(ck)


def test_scan_rejects_no_points():
    with pytest.raises(ValueError):
        scan_mod.scan(np.zeros((2, 2)), [], time_steps=4, warmup=1, sweeps=1)
