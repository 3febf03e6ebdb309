"""Unequal-time Green's function G(tau_l, 0) measured on the device (measure_tau=True):
pinned to the reference's non-interacting G(tau) (tools.compute_pole_gf_tau), checked
against the float64 oracle at U = 4, and stable at large beta."""
import numpy as np
import pytest
from scipy.linalg import expm

from conftest import golden
from latticeqmc_gb300 import ChainSpec, Engine, HubbardModel
from latticeqmc_gb300._native import LqmcError
from oracle import dqmc

pytestmark = pytest.mark.gpu

# the kernels' G(tau) is float64 whatever the sweep's precision
ENGINES = [("smem", "fp64"), ("tiled", "fp64"), ("tiled", "fp64e")]


def _square(side):
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(side)
    return m.ham_kinetic()


def _b(spec, field, l, sigma):
    return dqmc.exp_v_diag(field[:, l], spec.lamb, sigma)[:, None] * spec.exp_k


@pytest.mark.parametrize("engine,precision", ENGINES)
@pytest.mark.parametrize("side,stab", [(2, 4), (4, 8)])
def test_u0_matches_reference_pole_formula(engine, precision, side, stab):
    """At U = 0 every measured sample is -compute_pole_gf_tau(K, beta) at tau_l; at 4x4 with
    beta = 8 the products span exp(+-32), so this also checks the stabilisation."""
    f = golden("u0_gtau.npz")
    K, beta, L = f[f"s{side}_kinetic"], float(f[f"s{side}_beta"]), int(f[f"s{side}_L"])
    n = side * side
    spec = ChainSpec(K, 0.0, beta, L, np.ones((n, L), np.int8))
    eng = Engine([spec], mode="dqmc", precision=precision, engine=engine, rng="philox", seed=2,
                 stab_every=stab, measure_tau=True)
    eng.sweep(1)
    eng.sweep(3, measure=True)
    s, cnt = eng.green_tau_sum(0)
    assert cnt == 3
    assert eng.status()[0] == 0
    for sp in range(2):
        assert np.abs(s[sp] / cnt - f[f"s{side}_gtau"]).max() < 1e-10
    eng.close()


@pytest.mark.parametrize("engine,precision", ENGINES)
def test_matches_oracle_at_u4(engine, precision):
    """Each measured sample equals the oracle's G(tau_l, 0) of the field the sweep ended with
    (4x4, U = 4, beta = 2, L = 20: plain float64 products are accurate there)."""
    K = _square(4)
    rng = np.random.default_rng(7)
    spec = ChainSpec(K, 4.0, 2.0, 20, (2 * rng.integers(0, 2, (16, 20)) - 1).astype(np.int8))
    eng = Engine([spec], mode="dqmc", precision=precision, engine=engine, rng="philox", seed=9,
                 stab_every=5, measure_tau=True)
    eng.sweep(2)
    want = np.zeros((2, 20, 16, 16))
    for _ in range(3):
        eng.sweep(1, measure=True)
        field = eng.field(0)
        for sp, sigma in ((0, 1), (1, -1)):
            want[sp] += dqmc.green_tau(spec.exp_k, spec.lamb, field, sigma)
    s, cnt = eng.green_tau_sum(0)
    assert cnt == 3
    assert np.abs(s - want).max() < 1e-10 * cnt
    eng.close()


@pytest.mark.parametrize("engine,precision", ENGINES)
def test_measuring_tau_leaves_the_chain_unchanged(engine, precision):
    """With measure_tau the sweeps run one per launch (each followed by the G(tau) kernel);
    decisions, fields, G and every equal-time sum stay bit-identical, with replayed uniforms
    (indexed across the launches) and with Philox."""
    K = _square(4)
    rng = np.random.default_rng(3)
    specs = [ChainSpec(K, u, 2.0, 20, (2 * rng.integers(0, 2, (16, 20)) - 1).astype(np.int8))
             for u in (2.0, 4.0)]
    uni = rng.random((2, 3, 16 * 20))
    for rng_kind in ("replay", "philox"):
        runs = []
        for tau in (False, True):
            eng = Engine(specs, mode="dqmc", precision=precision, engine=engine, rng=rng_kind,
                         seed=4, stab_every=5, record=True, measure_tau=tau)
            if rng_kind == "replay":
                eng.set_uniforms_all(uni.reshape(-1))
            eng.sweep(3, measure=True)
            runs.append([(eng.decisions(c), eng.field(c), eng.green(c), eng.green_sum(c)[0],
                          eng.observables_raw(c)) for c in range(2)])
            if tau:
                assert eng.launch_count() == 6
            eng.close()
        for a, b in zip(*runs):
            for x, y in zip(a, b):
                assert np.array_equal(x, y)


def test_large_beta_antiperiodic_and_continuous():
    """6x6, U = 4, beta = 8 (L = 80): B_{L-1} G(tau_{L-1}, 0) = 1 - G(0) (antiperiodicity,
    from two independent stable recomputes), and at every recompute point the recomputed
    G(tau_c, 0) continues the propagated B_{c-1} G(tau_{c-1}, 0)."""
    K = _square(6)
    rng = np.random.default_rng(11)
    L, stab = 80, 10
    spec = ChainSpec(K, 4.0, 8.0, L, (2 * rng.integers(0, 2, (36, L)) - 1).astype(np.int8))
    eng = Engine([spec], mode="dqmc", precision="fp64", rng="philox", seed=5, stab_every=stab,
                 measure_tau=True)
    eng.sweep(5)
    eng.sweep(1, measure=True)
    g, cnt = eng.green_tau_sum(0)
    assert cnt == 1
    field = eng.field(0)
    for sp, sigma in ((0, 1), (1, -1)):
        x = g[sp]
        end = _b(spec, field, L - 1, sigma) @ x[L - 1]
        assert np.abs(end - (np.eye(36) - x[0])).max() < 1e-8
        for c in range(1, L // stab):
            l = c * stab
            prop = _b(spec, field, l - 1, sigma) @ x[l - 1]
            assert np.abs(prop - x[l]).max() < 1e-8
    eng.close()


def test_u0_wide_lattice_global_scratch():
    """12x12 (N = 144, scratch in global memory, GEMM columns in two blocks) at U = 0 against
    G(tau, 0) = V exp(-tau e) (1 + exp(-beta e))^-1 V^T from the eigenpairs of K."""
    K = _square(12)
    beta, L, stab = 4.0, 32, 8
    spec = ChainSpec(K, 0.0, beta, L, np.ones((144, L), np.int8))
    eng = Engine([spec], mode="dqmc", precision="fp64", engine="tiled", rng="philox", seed=1,
                 stab_every=stab, measure_tau=True)
    eng.sweep(1, measure=True)
    g, cnt = eng.green_tau_sum(0)
    e, v = np.linalg.eigh(K)
    for l in range(L):
        tau = l * beta / L
        want = (v * (np.exp(-tau * e) / (1.0 + np.exp(-beta * e)))) @ v.T
        assert np.abs(g[0, l] - want).max() < 1e-9
        assert np.abs(g[1, l] - want).max() < 1e-9
    eng.close()


def test_checkpoint_carries_the_tau_sums(tmp_path):
    K = _square(4)
    rng = np.random.default_rng(2)
    specs = [ChainSpec(K, 4.0, 2.0, 20, (2 * rng.integers(0, 2, (16, 20)) - 1).astype(np.int8))]
    kw = dict(mode="dqmc", precision="fp64", rng="philox", seed=3, stab_every=5, measure_tau=True)
    straight = Engine(specs, **kw)
    straight.sweep(4, measure=True)
    ref = straight.green_tau_sum(0)[0]
    straight.close()
    first = Engine(specs, **kw)
    first.sweep(2, measure=True)
    first.checkpoint(tmp_path / "ck.npz")
    first.close()
    second = Engine(specs, **kw)
    second.restore(tmp_path / "ck.npz")
    second.sweep(2, measure=True)
    assert np.array_equal(second.green_tau_sum(0)[0], ref)
    second.close()


def test_tau_sums_need_measure_tau():
    K = _square(2)
    eng = Engine([ChainSpec(K, 4.0, 1.0, 10, np.ones((4, 10), np.int8))], mode="dqmc",
                 rng="philox", stab_every=5)
    eng.sweep(1, measure=True)
    with pytest.raises(LqmcError):
        eng.green_tau_sum(0)
    eng.close()
    with pytest.raises(LqmcError):
        Engine([ChainSpec(K, 4.0, 1.0, 10, np.ones((4, 10), np.int8))], mode="compat",
               rng="philox", measure_tau=True)
