"""The alternating sweep order (sweeps down and up in turn) on the GPU against the oracle's
alternating sweeps (oracle/dqmc.py, Chain.sweep_alternating), and its physics against the
exact diagonalisation."""
import numpy as np
import pytest
from scipy.linalg import expm

from latticeqmc_gb300 import ChainSpec, Engine, HubbardModel
from oracle import dqmc as odqmc
from oracle import ed

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-8, "fp64e": 1e-6}


def _lattice(side):
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(side)
    return m.ham_kinetic()


@pytest.mark.parametrize("side,beta,L,stab,sweeps,precision",
                         [(4, 4.0, 40, 8, 4, "fp64"), (4, 4.0, 40, 8, 4, "fp64e"),
                          (8, 4.0, 40, 10, 3, "fp64e"), (16, 8.0, 80, 8, 2, "fp64"),
                          (16, 8.0, 80, 8, 3, "fp64e")])
def test_alternating_order_matches_oracle(side, beta, L, stab, sweeps, precision):
    K = _lattice(side)
    n = side * side
    rng = np.random.default_rng(700 + side)
    field = (2 * rng.integers(0, 2, (n, L)) - 1).astype(np.int8)
    spec = ChainSpec(K, 4.0, beta, L, field)
    ch = odqmc.Chain(spec.exp_k, expm(spec.dtau * K), spec.lamb, field, stab)
    eng = Engine([spec], mode="dqmc", precision=precision, rng="replay", record=True,
                 stab_every=stab, sweep_order="alternate")
    try:
        for sw in range(sweeps):
            u = rng.random(n * L)
            rec = {}
            g_or = ch.sweep_alternating(u, record=rec)
            eng.set_uniforms(0, u)
            eng.sweep(1)
            dec = eng.decisions(0)[0]
            assert np.array_equal(dec, rec["accept"]), (
                f"sweep {sw}: {int((dec != rec['accept']).sum())} decisions differ")
            dg = float(np.abs(eng.green(0) - g_or).max())
            d = eng.diagnostics(0)
            print(f"alternate {precision} {side}x{side} sweep {sw} ({'down' if sw % 2 == 0 else 'up'}): "
                  f"max|dG| {dg:.2e}, residual {d['max_residual']:.1e} (oracle {ch.max_resid:.1e})")
            assert dg < TOL[precision]
            assert d["sweeps"] == sw + 1
            np.testing.assert_allclose(d["logdet"], ch.logdet, rtol=1e-9, atol=1e-7)
            np.testing.assert_array_equal(eng.field(0), ch.field)
        assert not (eng.status() & 11).any()
    finally:
        eng.close()


def test_alternating_order_restarts_from_scratch_after_set_field():
    """A new field invalidates the products kept between sweeps: the next sweep goes down
    from a fresh right stack, exactly like a new engine's first sweep."""
    K = _lattice(4)
    rng = np.random.default_rng(9)
    f1 = (2 * rng.integers(0, 2, (16, 40)) - 1).astype(np.int8)
    f2 = (2 * rng.integers(0, 2, (16, 40)) - 1).astype(np.int8)
    u = rng.random(3 * 16 * 40)
    a = Engine([ChainSpec(K, 4.0, 4.0, 40, f1)], mode="dqmc", rng="replay", record=True,
               stab_every=8, sweep_order="alternate")
    b = Engine([ChainSpec(K, 4.0, 4.0, 40, f2)], mode="dqmc", rng="replay", record=True,
               stab_every=8, sweep_order="alternate")
    try:
        a.set_uniforms(0, u[:2 * 640])
        a.sweep(2)                      # down, up: the next would go down on kept products
        a.set_field(0, f2)
        a.set_uniforms(0, u[2 * 640:])
        a.sweep(1)
        b.set_uniforms(0, u[2 * 640:])
        b.sweep(1)
        np.testing.assert_array_equal(a.decisions(0), b.decisions(0))
        np.testing.assert_array_equal(a.green(0), b.green(0))
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("precision", ["fp64", "fp64e"])
def test_alternating_order_2x2_observables_match_exact_diagonalisation(precision):
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(2)
    K = m.ham_kinetic()
    rng = np.random.default_rng(22)
    U, beta, L, n_chains = 4.0, 2.0, 20, 64
    specs = [ChainSpec(K, U, beta, L, (2 * rng.integers(0, 2, (4, L)) - 1).astype(np.int8))
             for _ in range(n_chains)]
    eng = Engine(specs, mode="dqmc", precision=precision, rng="philox", seed=31, stab_every=5,
                 sweep_order="alternate")
    eng.sweep(200)
    eng.reset_measurements()
    eng.sweep(1000, measure=True)
    obs = [eng.observables(c) for c in range(n_chains)]
    assert not (eng.status() & 11).any()
    eng.close()
    exact = ed.observables(K, U, beta, L)
    for key, ref in (("double_occupancy_mean", exact["double_occupancy"].mean()),
                     ("kinetic_energy", exact["kinetic_energy"]),
                     ("potential_energy", exact["potential_energy"])):
        vals = np.array([o[key] for o in obs])
        mean, err = vals.mean(), vals.std(ddof=1) / np.sqrt(n_chains)
        print(f"alternate {precision} {key}: {mean:.5f} +- {err:.5f} vs ED {ref:.5f}")
        assert abs(mean - ref) < 4 * err + 1e-4, f"{key}: {mean:.5f} +- {err:.5f} vs ED {ref:.5f}"
