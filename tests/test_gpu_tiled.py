"""The tiled kernel (matrices in global memory, block-tiled GEMMs) in float64 and in mixed
precision, against the CPU oracle and against the shared-memory kernel."""
import numpy as np
import pytest
from scipy.linalg import expm

from latticeqmc_gb300 import ChainSpec, Engine, HubbardModel, _native
from oracle import dqmc as odqmc
from oracle import ed

pytestmark = pytest.mark.gpu


def _status_matches_residual(eng, bound=None):
    """After one sweep(1) call: no bit but LQMC_STATUS_DRIFT, and DRIFT set exactly when the
    call's largest stabilisation residual exceeds the 1e-6 drift threshold (float32 G, or
    the emulated products' last bits amplified by the wraps, can pass it by design); with
    `bound`, the residual itself stays below it."""
    st = int(eng.status()[0])
    resid = eng.diagnostics(0)["max_residual"]
    print(f"status {st}, max residual {resid:.2e}")
    assert st & ~_native.STATUS_DRIFT == 0
    assert bool(st & _native.STATUS_DRIFT) == (resid > 1e-6)
    if bound is not None:
        assert resid < bound

def _setup(side, beta, L, seed, u=4.0):
    m = HubbardModel(u=u, t=1, mu=0)
    m.build_square(side)
    K = m.ham_kinetic()
    rng = np.random.default_rng(seed)
    field = (2 * rng.integers(0, 2, (side * side, L)) - 1).astype(np.int8)
    return K, field, rng


@pytest.mark.parametrize("side,beta,L,stab", [(2, 2.0, 20, 5), (4, 4.0, 40, 5), (6, 4.0, 40, 5),
                                              (8, 4.0, 80, 10), (12, 4.0, 40, 5)])
def test_tiled_fp64_matches_oracle(side, beta, L, stab):
    K, field, rng = _setup(side, beta, L, 300 + side)
    N = side * side
    spec = ChainSpec(K, 4.0, beta, L, field)
    ch = odqmc.Chain(spec.exp_k, expm(spec.dtau * K), spec.lamb, field, stab)
    eng = Engine([spec], mode="dqmc", rng="replay", record=True, stab_every=stab, engine="tiled")
    for sw in range(2 if N <= 64 else 1):
        u = rng.random(N * L)
        rec = {}
        g_or = ch.sweep(u, record=rec)
        eng.set_uniforms(0, u)
        eng.sweep(1)
        assert np.array_equal(eng.decisions(0)[0], rec["accept"])
        assert np.abs(eng.green(0) - g_or).max() < 1e-10
        d = eng.diagnostics(0)
        np.testing.assert_allclose(d["logdet"], ch.logdet, rtol=1e-9, atol=1e-9)
    assert not eng.status().any()
    eng.close()


def test_tiled_and_smem_kernels_agree():
    K, field, rng = _setup(8, 4.0, 40, 5)
    spec = ChainSpec(K, 4.0, 4.0, 40, field)
    a = Engine([spec], mode="dqmc", rng="philox", seed=9, stab_every=5, engine="smem", record=True)
    b = Engine([spec], mode="dqmc", rng="philox", seed=9, stab_every=5, engine="tiled", record=True)
    a.sweep(3, measure=True)
    b.sweep(3, measure=True)
    np.testing.assert_array_equal(a.decisions(0), b.decisions(0))
    assert np.abs(a.green(0) - b.green(0)).max() < 1e-10
    np.testing.assert_allclose(a.observables_raw(0), b.observables_raw(0), atol=1e-8)
    a.close()
    b.close()


def test_tiled_u0_known_answer_large_lattice():
    K, field, _ = _setup(12, 4.0, 40, 1, u=0.0)
    eng = Engine([ChainSpec(K, 0.0, 4.0, 40, field)], mode="dqmc", rng="philox")
    eng.sweep(1)
    w, v = np.linalg.eigh(K)
    exact = (v * (0.5 * (1.0 + np.tanh(0.5 * 4.0 * w)))) @ v.T
    assert np.abs(eng.green(0)[0] - exact).max() < 1e-10
    eng.close()


@pytest.mark.parametrize("side,beta,L,stab", [(4, 4.0, 40, 8), (8, 4.0, 40, 8)])
def test_mixed_precision_against_fp64(side, beta, L, stab):
    """Same field and uniforms: the float32 engine's G after one sweep against the float64
    engine's.  Float32 rounding of G is amplified by the wraps between refreshes (up to
    e^{stab dtau (8t + 2 lambda)}), so the bar is the measured float32 drift, not 1e-10."""
    K, field, rng = _setup(side, beta, L, 40 + side)
    N = side * side
    spec = ChainSpec(K, 4.0, beta, L, field)
    f64 = Engine([spec], mode="dqmc", rng="replay", stab_every=stab, record=True)
    f32 = Engine([spec], mode="dqmc", precision="mixed", rng="replay", stab_every=stab, record=True)
    u = rng.random(N * L)
    f64.set_uniforms(0, u)
    f32.set_uniforms(0, u)
    f64.sweep(1)
    f32.sweep(1)
    same = np.array_equal(f64.decisions(0), f32.decisions(0))
    dg = np.abs(f64.green(0) - f32.green(0)).max()
    print(f"mixed vs fp64 {side}x{side}: decisions identical {same}, max|dG| {dg:.2e}")
    if same:
        assert dg < 2e-2
    _status_matches_residual(f32)


def test_mixed_precision_2x2_observables_match_exact_diagonalisation():
    K, _, rng = _setup(2, 2.0, 20, 0)
    U, beta, L, n_chains = 4.0, 2.0, 20, 64
    specs = [ChainSpec(K, U, beta, L, (2 * rng.integers(0, 2, (4, L)) - 1).astype(np.int8))
             for _ in range(n_chains)]
    eng = Engine(specs, mode="dqmc", precision="mixed", rng="philox", seed=77, stab_every=5)
    eng.sweep(200)
    eng.reset_measurements()
    eng.sweep(1000, measure=True)
    obs = [eng.observables(c) for c in range(n_chains)]
    eng.close()
    exact = ed.observables(K, U, beta, L)
    for key, ref in (("double_occupancy_mean", exact["double_occupancy"].mean()),
                     ("kinetic_energy", exact["kinetic_energy"]),
                     ("potential_energy", exact["potential_energy"])):
        vals = np.array([o[key] for o in obs])
        mean, err = vals.mean(), vals.std(ddof=1) / np.sqrt(n_chains)
        assert abs(mean - ref) < 4 * err + 1e-4, f"{key}: {mean:.5f} +- {err:.5f} vs ED {ref:.5f}"


@pytest.mark.parametrize("side,beta,L,stab", [(4, 4.0, 40, 5), (8, 4.0, 80, 10), (12, 4.0, 40, 5)])
def test_fp64e_matches_oracle(side, beta, L, stab):
    """Every dense product on the BF16 tensor cores, operands carried as 55-bit fixed-point
    integers in eight BF16 digits: decisions as the float64 oracle, G within the
    wrap-amplified rounding error (1e-8)."""
    K, field, rng = _setup(side, beta, L, 500 + side)
    N = side * side
    spec = ChainSpec(K, 4.0, beta, L, field)
    ch = odqmc.Chain(spec.exp_k, expm(spec.dtau * K), spec.lamb, field, stab)
    eng = Engine([spec], mode="dqmc", precision="fp64e", rng="replay", record=True, stab_every=stab)
    for sw in range(2 if N <= 64 else 1):
        u = rng.random(N * L)
        rec = {}
        g_or = ch.sweep(u, record=rec)
        eng.set_uniforms(0, u)
        eng.sweep(1)
        assert np.array_equal(eng.decisions(0)[0], rec["accept"])
        dg = np.abs(eng.green(0) - g_or).max()
        print(f"fp64e vs oracle {side}x{side}: max|dG| {dg:.2e}")
        assert dg < 1e-8
    assert not eng.status().any()
    eng.close()


def test_fp64e_against_fp64_engine_16x16_beta8():
    """The headline configuration's lattice: identical inputs, one sweep, max|dG| <= 1e-6."""
    K, field, rng = _setup(16, 8.0, 80, 16)
    spec = ChainSpec(K, 4.0, 8.0, 80, field)
    a = Engine([spec], mode="dqmc", precision="fp64", rng="replay", stab_every=8, record=True)
    b = Engine([spec], mode="dqmc", precision="fp64e", rng="replay", stab_every=8, record=True)
    u = rng.random(256 * 80)
    a.set_uniforms(0, u)
    b.set_uniforms(0, u)
    a.sweep(1)
    b.sweep(1)
    assert np.array_equal(a.decisions(0), b.decisions(0))
    dg = np.abs(a.green(0) - b.green(0)).max()
    print(f"fp64e vs fp64 16x16 beta=8: max|dG| {dg:.2e}, residual {b.diagnostics(0)['max_residual']:.1e}")
    assert dg < 1e-6
    _status_matches_residual(b, bound=1e-5)
    a.close()
    b.close()


def test_fp64e_batched_chains_match_single_chain_runs():
    """Chains of several sizes in one launch (one bucket per size, one CTA pair per chain)
    give bit-identical G to the same chains run alone."""
    specs, us = [], []
    for side, seed in ((4, 1), (6, 2), (10, 3), (6, 4)):
        K, field, rng = _setup(side, 2.0, 20, 900 + seed)
        specs.append(ChainSpec(K, 4.0, 2.0, 20, field))
        us.append(rng.random(side * side * 20))
    both = Engine(specs, mode="dqmc", precision="fp64e", rng="replay", stab_every=5)
    both.set_uniforms_all(np.concatenate(us))
    both.sweep(1)
    for c, (spec, u) in enumerate(zip(specs, us)):
        one = Engine([spec], mode="dqmc", precision="fp64e", rng="replay", stab_every=5)
        one.set_uniforms(0, u)
        one.sweep(1)
        assert np.array_equal(one.green(0), both.green(c))
        one.close()
    assert not both.status().any()
    both.close()


def test_fp64e_stalled_tensor_core_wait_reports_timeout():
    """The tensor-core pipeline's waits are bounded: with the test hook that issues no
    copies for the first step, the wait runs out (about a second), the chain reports
    LQMC_STATUS_TIMEOUT, and the context stays usable for the next handle."""
    from latticeqmc_gb300 import _native
    K, field, rng = _setup(8, 2.0, 20, 77)
    spec = ChainSpec(K, 4.0, 2.0, 20, field)
    bad = Engine([spec], mode="dqmc", precision="fp64e", rng="philox", seed=3, stab_every=5,
                 debug=_native.DEBUG_STALL_TC_WAIT)
    bad.sweep(1)
    st = bad.status()
    assert st[0] & _native.STATUS_TIMEOUT
    bad.close()
    good = Engine([spec], mode="dqmc", precision="fp64e", rng="philox", seed=3, stab_every=5)
    good.sweep(2)
    assert not good.status().any()
    assert np.isfinite(good.green(0)).all()
    good.close()


def test_fp64e_with_every_category_native_is_the_fp64_engine():
    """Routing every product category of the fp64e engine to native float64 reproduces the
    plain float64 tiled engine bit for bit (same kernel code, only the GEMMs differ)."""
    K, field, rng = _setup(10, 4.0, 40, 31)
    spec = ChainSpec(K, 4.0, 4.0, 40, field)
    u = rng.random(100 * 40)
    a = Engine([spec], mode="dqmc", precision="fp64", engine="tiled", rng="replay", stab_every=5,
               delay=16)
    b = Engine([spec], mode="dqmc", precision="fp64e", rng="replay", stab_every=5, delay=16,
               fp64e_native=("wrap", "stack", "udt", "green", "update", "lu", "lu_rhs"))
    for e in (a, b):
        e.set_uniforms(0, u)
        e.sweep(1)
    assert np.array_equal(a.green(0), b.green(0))
    a.close()
    b.close()
