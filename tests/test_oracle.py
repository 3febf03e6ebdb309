"""Pin the CPU oracle against the reference's recorded outputs and known answers (CPU only)."""
import itertools

import numpy as np
import pytest
from scipy.linalg import expm

from conftest import golden, kinetic_from_golden
from oracle import compat, dqmc, ed, philox


@pytest.mark.parametrize("side,n_sweeps", [(2, None), (4, None), (8, 1)])
def test_compat_oracle_bit_identical_to_reference(side, n_sweeps):
    f = golden(f"compat_{side}x{side}.npz")
    field = f["field0"].copy()
    N, L = field.shape
    u = f["uniforms"]
    for sw in range(n_sweeps or int(f["n_sweeps"])):
        rec = {}
        g = compat.update_step(f["exp_k"], field, float(f["lamb"]), u[sw * N * L:(sw + 1) * N * L],
                               record=rec)
        np.testing.assert_array_equal(rec["accept"], f["accept"][sw])
        np.testing.assert_array_equal(rec["ratio"], f["ratio"][sw])
        np.testing.assert_array_equal(np.stack(g), f["green"][sw])
    if n_sweeps is None:
        np.testing.assert_array_equal(field, f["field_end"])


def test_compat_loop_and_outer_rank1_identical():
    f = golden("compat_2x2.npz")
    N, L = f["field0"].shape
    u = f["uniforms"][:N * L]
    a = compat.update_step(f["exp_k"], f["field0"].copy(), float(f["lamb"]), u, rank1="loop")
    b = compat.update_step(f["exp_k"], f["field0"].copy(), float(f["lamb"]), u, rank1="outer")
    np.testing.assert_array_equal(np.stack(a), np.stack(b))


def test_compat_run_matches_reference_run():
    f = golden("run_2x2.npz")
    g = compat.run(f["exp_k"], f["field0"].copy(), float(f["lamb"]), f["uniforms"],
                   int(f["warmup"]), int(f["sweeps"]))
    np.testing.assert_array_equal(g, f["green_mean"])


def test_compat_set_beta_and_constants_match_reference():
    f = golden("compat_4x4.npz")
    dtau, lamb, exp_k = compat.set_beta(f["kinetic"], float(f["u"]), float(f["beta"]), int(f["L"]))
    assert lamb == float(f["lamb"])
    np.testing.assert_array_equal(exp_k, f["exp_k"])
    np.testing.assert_array_equal(compat.exp_constants(lamb, 16), f["consts"])


def test_diag_product_is_exact_scaling():
    """np.dot(exp_k, diagflat(d)) equals the column scaling exp_k * d bit for bit, which the
    device uses in place of the dense product (lqmc.py:182, :341)."""
    f = golden("compat_8x8.npz")
    ek = f["exp_k"]
    d = np.exp(-float(f["lamb"]) * f["field0"][:, 3].astype(np.float64))
    np.testing.assert_array_equal(np.dot(ek, np.diagflat(d)), ek * d[None, :])
    np.testing.assert_array_equal(np.dot(np.diagflat(d), ek), d[:, None] * ek)


@pytest.mark.parametrize("name", ["det_2x2.npz", "det_4x4.npz"])
def test_dqmc_ratios_equal_reference_determinant_ratios(name):
    f = golden(name)
    N, L = f["field0"].shape
    ch = dqmc.Chain(f["exp_k"], f["exp_k_inv"], float(f["lamb"]), f["field0"], stab_every=5)
    u = f["uniforms"]
    for sw in range(int(f["n_sweeps"])):
        rec = {}
        ch.sweep(u[sw * N * L:(sw + 1) * N * L], record=rec)
        np.testing.assert_array_equal(rec["accept"], f["accept"][sw])
        np.testing.assert_allclose(rec["ratio"], f["ratio"][sw], rtol=1e-9)
    np.testing.assert_array_equal(ch.field, f["field_end"])


def test_dqmc_u0_known_answer():
    f = golden("u0_known.npz")
    for side in (2, 4):
        K, beta, L = f[f"s{side}_kinetic"], float(f[f"s{side}_beta"]), int(f[f"s{side}_L"])
        dt = beta / L
        field = np.ones((side * side, L), np.int8)
        ch = dqmc.Chain(expm(-dt * K), expm(dt * K), 0.0, field, stab_every=5)
        g = ch.sweep(np.random.default_rng(0).random(side * side * L))
        assert np.abs(g[0] - f[f"s{side}_pole_tau0"]).max() < 1e-12
        assert np.abs(g[1] - f[f"s{side}_pole_tau0"]).max() < 1e-12


def test_green_tau_oracle_u0_known_answer():
    """The oracle's unequal-time G at U = 0 against the reference's compute_pole_gf_tau
    (tools.py:182-200) at the slice times; beta = 2, where plain products are exact."""
    f = golden("u0_gtau.npz")
    K, beta, L = f["s2_kinetic"], float(f["s2_beta"]), int(f["s2_L"])
    field = np.ones((4, L), np.int8)
    for sigma in (1, -1):
        g = dqmc.green_tau(expm(-beta / L * K), 0.0, field, sigma)
        assert np.abs(g - f["s2_gtau"]).max() < 1e-13


def test_green_tau_oracle_relations_to_equal_time_green():
    """The end-of-sweep G of the chain (the equal-time G at tau_1) times B_0 is G(tau_1, 0),
    and B_{L-1} G(tau_{L-1}, 0) = B(beta, 0) G(0) = 1 - G(0)."""
    K = kinetic_from_golden(4)
    beta, L, U = 2.0, 20, 4.0
    dt = beta / L
    lamb = np.arccosh(np.exp(U * dt / 2))
    rng = np.random.default_rng(5)
    field = (2 * rng.integers(0, 2, (16, L)) - 1).astype(np.int8)
    ch = dqmc.Chain(expm(-dt * K), expm(dt * K), lamb, field.copy(), stab_every=5)
    ch.sweep(np.full(16 * L, np.inf))       # u = inf rejects every flip: the field stays
    assert (ch.field == field).all()
    for s, sigma in ((0, 1), (1, -1)):
        g = dqmc.green_tau(expm(-dt * K), lamb, field, sigma)
        b = [dqmc.exp_v_diag(field[:, l], lamb, sigma)[:, None] * expm(-dt * K) for l in range(L)]
        assert np.abs(ch.green[s] @ b[0] - g[1]).max() < 1e-11
        assert np.abs(b[L - 1] @ g[L - 1] - (np.eye(16) - g[0])).max() < 1e-11


def test_dqmc_stabilisation_residual_small_at_large_beta():
    K = kinetic_from_golden(8)
    beta, L, U = 10.0, 100, 4.0
    dt = beta / L
    lamb = np.arccosh(np.exp(U * dt / 2))
    rng = np.random.default_rng(1)
    field = (2 * rng.integers(0, 2, (64, L)) - 1).astype(np.int8)
    ch = dqmc.Chain(expm(-dt * K), expm(dt * K), lamb, field, stab_every=5)
    ch.sweep(rng.random(64 * L))
    assert ch.max_resid < 1e-8


def test_estimator_equals_exact_diagonalisation_by_enumeration():
    """Sum over all 2^(N L) HS fields of a 2x2, L=3 lattice: the weighted mean of the
    engine's Green's-function estimator and Wick measurements equals the Trotterised ED."""
    K = kinetic_from_golden(2)
    U, beta, L, N = 4.0, 1.0, 3, 4
    dt = beta / L
    lamb = np.arccosh(np.exp(U * dt / 2))
    ek = expm(-dt * K)
    wsum, gacc, ekin, docc = 0.0, np.zeros((2, N, N)), 0.0, 0.0
    for bits in itertools.product((1, -1), repeat=N * L):
        s = np.array(bits, dtype=np.int8).reshape(N, L)
        ch = dqmc.Chain(ek, expm(dt * K), lamb, s, stab_every=2)
        gs, w = [], 1.0
        for sig in (1, -1):
            stack = ch.right_stack(sig)
            # G~_0 = (1 + B_0 B_{L-1} ... B_1): wrap the fresh G~_{L-1} down to slice 0
            g, logdet, sgn = dqmc.green_from_udt(stack[-1], dqmc.identity_udt(N))
            for l in range(L - 1, 0, -1):
                g = ch.wrap(l, g, sig)
            gs.append(g)
            w *= sgn * np.exp(-logdet)
        o = dqmc.measure(np.array(gs), K, U)
        wsum += w
        gacc += w * np.array(gs)
        ekin += w * o["kinetic_energy"]
        docc += w * o["double_occupancy"].mean()
    ex = ed.observables(K, U, beta, L)
    assert abs(ekin / wsum - ex["kinetic_energy"]) < 1e-10
    assert abs(docc / wsum - ex["double_occupancy"].mean()) < 1e-10
    assert np.abs(gacc / wsum - ex["green"]).max() < 1e-10


def test_ed_u0_is_free_fermions():
    K = kinetic_from_golden(2)
    beta, L = 2.0, 10
    ex = ed.observables(K, 0.0, beta, L)
    exact = np.linalg.inv(np.eye(4) + expm(-beta * K))
    np.testing.assert_allclose(ex["green"][0], exact, atol=1e-12)
    np.testing.assert_allclose(ex["density"], 1.0, atol=1e-12)


def test_philox_matches_numpy_philox():
    for ctr, key in (((0, 0, 0, 0), (0, 0)), ((5, 7, 1, 2), (123, 4)),
                     ((2 ** 64 - 2, 3, 0, 0), (2 ** 63, 17))):
        bg = np.random.Philox(counter=np.array(ctr, dtype=np.uint64), key=np.array(key, dtype=np.uint64))
        raw = [int(x) for x in bg.random_raw(4)]
        nxt = ((ctr[0] + 1) % 2 ** 64, ctr[1] + (ctr[0] + 1) // 2 ** 64, ctr[2], ctr[3])
        assert raw == philox.philox4x64(nxt, key)


def test_philox_uniforms_in_unit_interval_and_distinct_streams():
    a = philox.uniforms(1, 0, 0, 16, 20)
    b = philox.uniforms(1, 1, 0, 16, 20)
    c = philox.uniforms(1, 0, 1, 16, 20)
    assert a.min() >= 0.0 and a.max() < 1.0
    assert not np.array_equal(a, b) and not np.array_equal(a, c)
    assert abs(np.concatenate([a, b, c]).mean() - 0.5) < 0.05


def test_green_tau_oracle_matches_reference_exact_chain():
    """The reference's own U = 0 validation (exact.py:37-54): a 10-site open chain at beta = 4,
    G(tau_l, 0) against its compute_pole_gf_tau at the 32 slice times."""
    f = golden("exact_chain10_gtau.npz")
    K, beta, L = f["kinetic"], float(f["beta"]), int(f["L"])
    field = np.ones((K.shape[0], L), np.int8)
    for sigma in (1, -1):
        g = dqmc.green_tau(expm(-beta / L * K), 0.0, field, sigma)
        assert np.abs(g - f["gtau"]).max() < 1e-12


@pytest.mark.parametrize("L,stabs", [(23, (1, 5, 23)), (7, (1, 3, 4))])
def test_dqmc_ragged_refresh_chunks_agree(L, stabs):
    """A slice count the refresh interval does not divide (a shorter last chunk) gives the same
    decisions and G as refreshing every slice, and as one chunk for the whole sweep."""
    K = kinetic_from_golden(2)
    dt, U = 0.05, 4.0
    lamb = np.arccosh(np.exp(U * dt / 2))
    rng = np.random.default_rng(L)
    field = (2 * rng.integers(0, 2, (4, L)) - 1).astype(np.int8)
    uni = rng.random(3 * 4 * L)
    runs = []
    for stab in stabs:
        ch = dqmc.Chain(expm(-dt * K), expm(dt * K), lamb, field.copy(), stab_every=stab)
        out = []
        for sw in range(3):
            rec = {}
            g = ch.sweep(uni[sw * 4 * L:(sw + 1) * 4 * L], record=rec)
            out.append((rec["accept"].copy(), np.array(g)))
        runs.append((out, ch.field.copy()))
    (ref, f_ref), others = runs[0], runs[1:]
    for out, f in others:
        np.testing.assert_array_equal(f, f_ref)
        for (acc, g), (acc0, g0) in zip(out, ref):
            np.testing.assert_array_equal(acc, acc0)
            assert np.abs(g - g0).max() < 1e-11


def _square(side):
    if side in (2, 4):
        return kinetic_from_golden(side)
    from latticeqmc_gb300 import HubbardModel
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(side)
    return m.ham_kinetic()


def test_alternating_sweeps_keep_g_equal_to_a_fresh_recompute():
    """Sweeps down and up in turn: after every sweep G equals (1 + B_{L-1} .. B_0)^-1 of the
    field as it now stands, computed from scratch, and the refreshes agree with the wraps."""
    K = _square(4)
    beta, L, stab, u = 4.0, 40, 8, 4.0
    dtau = beta / L
    lamb = np.arccosh(np.exp(u * dtau / 2.0))
    ek, eki = expm(-dtau * K), expm(dtau * K)
    rng = np.random.default_rng(11)
    field = (2 * rng.integers(0, 2, (16, L)) - 1).astype(np.int8)
    ch = dqmc.Chain(ek, eki, lamb, field, stab)
    for sw in range(4):
        g = ch.sweep_alternating(rng.random(16 * L))
        ref = dqmc.Chain(ek, eki, lamb, ch.field, stab)
        for s, sigma in ((0, +1), (1, -1)):
            gs = dqmc.green_from_udt(ref.right_stack(sigma)[-1], dqmc.identity_udt(16))[0]
            assert np.abs(g[s] - gs).max() < 1e-12
        assert ch.max_resid < 1e-9
        assert ch.alt_state == (1 if sw % 2 == 0 else 2)


def test_alternating_up_sweep_ratios_are_determinant_ratios():
    """Every ratio of an up sweep (2x2, beta=1, L=10: small enough for plain determinants) is
    det M(flipped) / det M of the configuration the site saw: slices below already updated,
    its own slice updated up to the site, the rest as before the sweep."""
    K = _square(2)
    beta, L, stab, u = 1.0, 10, 4, 4.0
    dtau = beta / L
    lamb = np.arccosh(np.exp(u * dtau / 2.0))
    ek = expm(-dtau * K)
    rng = np.random.default_rng(5)
    field = (2 * rng.integers(0, 2, (4, L)) - 1).astype(np.int8)
    ch = dqmc.Chain(ek, expm(dtau * K), lamb, field, stab)
    ch.sweep_alternating(rng.random(4 * L))          # down
    before = ch.field.copy()
    rec = {}
    ch.sweep_alternating(rng.random(4 * L), record=rec)   # up

    def det_both(f):
        tot = 1.0
        for sigma in (+1, -1):
            m = np.eye(4)
            for ll in range(L):
                m = dqmc.exp_v_diag(f[:, ll], lamb, sigma)[:, None] * (ek @ m)
            tot *= np.linalg.det(np.eye(4) + m)
        return tot
    cfg = before.copy()
    for l in range(L):
        for i in range(4):
            fl = cfg.copy()
            fl[i, l] *= -1
            np.testing.assert_allclose(rec["ratio"][l, i], det_both(fl) / det_both(cfg), rtol=1e-10)
            if rec["accept"][l, i]:
                cfg = fl
    np.testing.assert_array_equal(cfg, ch.field)
