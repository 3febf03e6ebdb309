"""C-ABI behaviour on a GPU: error codes, state checks, health status, facade entry points."""
import ctypes

import numpy as np
import pytest

from latticeqmc_gb300 import ChainSpec, Engine, HubbardModel, LatticeQMC, measure, measure_betas
from latticeqmc_gb300 import _native

pytestmark = pytest.mark.gpu


def _k(side):
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(side)
    return m.ham_kinetic()


def test_error_codes():
    lib = _native.load()
    h = _native.Handle("dqmc", "fp64", "replay", 10, 0, 0, False, 0)
    # sweep before chains are defined
    assert lib.lqmc_sweep(h.h, 1, 0, None) == -3
    assert b"lqmc_set_chains" in lib.lqmc_last_error(h.h)
    h.close()
    spec = ChainSpec(_k(2), 4.0, 2.0, 20, np.ones((4, 20), np.int8))
    eng = Engine([spec], mode="dqmc", rng="replay")
    # replay mode without uniforms
    with pytest.raises(_native.LqmcError) as e:
        eng.sweep(1)
    assert e.value.code == -3
    # wrong uniform count
    with pytest.raises(_native.LqmcError) as e:
        eng.set_uniforms(0, np.zeros(7))
    assert e.value.code == -1
    # field values outside {-1, +1}
    with pytest.raises(_native.LqmcError) as e:
        eng.set_field(0, np.zeros((4, 20), np.int8))
    assert e.value.code == -1
    # chain index out of range
    out = np.zeros((2, 4, 4))
    assert lib.lqmc_get_green(eng._h.h, 1, _native.ptr(out)) == -1
    assert lib.lqmc_get_green(eng._h.h, -1, _native.ptr(out)) == -1
    eng.close()
    # lattices above the shared-memory kernel's limit: compat mode and engine="smem" refuse
    big = ChainSpec(np.zeros((200, 200)), 4.0, 1.0, 10, np.ones((200, 10), np.int8))
    with pytest.raises(_native.LqmcError) as e:
        Engine([big], mode="compat", rng="replay")
    assert e.value.code == -4
    with pytest.raises(_native.LqmcError) as e:
        Engine([big], mode="dqmc", engine="smem")
    assert e.value.code == -4
    # compat mode has no mixed-precision or tiled variant
    with pytest.raises(_native.LqmcError) as e:
        Engine([spec], mode="compat", precision="mixed", rng="replay")
    assert e.value.code == -4
    # bad enum in lqmc_create
    p = _native.Params(mode=7)
    hh = ctypes.c_void_p()
    assert lib.lqmc_create(ctypes.byref(p), ctypes.byref(hh)) == -1
    assert b"mode" in lib.lqmc_last_error(None)


def test_nonfinite_chain_is_flagged_not_fatal():
    """A chain fed a NaN in exp(-dtau K) reports LQMC_STATUS_NONFINITE; its neighbours in
    the same launch stay healthy."""
    K = _k(4)
    good = ChainSpec(K, 4.0, 2.0, 20, np.ones((16, 20), np.int8))
    bad_ek = good.exp_k.copy()
    bad_ek[3, 5] = np.nan
    bad = ChainSpec(K, 4.0, 2.0, 20, np.ones((16, 20), np.int8), exp_k=bad_ek)
    eng = Engine([good, bad, good], mode="dqmc", rng="philox", seed=1)
    eng.sweep(1)
    st = eng.status()
    assert st[0] == 0 and st[2] == 0
    assert st[1] & _native.STATUS_NONFINITE
    assert np.isfinite(eng.green(0)).all()
    eng.close()


def test_facade_single_chain_and_measure_entry_points():
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(2)
    np.random.seed(3)
    q = LatticeQMC(m, beta=2.0, time_steps=20, warmup=5, sweeps=10, log_lvl=None, mode="dqmc")
    g = q.run()
    assert g.shape == (2, 4, 4) and np.isfinite(g).all()
    gu, gd = q._update_step()
    assert gu.shape == (4, 4)
    o = q.observables()
    assert o["count"] == 10
    gu, gd = measure(m, 2.0, 20, 10, 40, cores=4, mode="dqmc", seed=1)
    assert gu.shape == (4, 4) and np.isfinite(gu).all()
    bu, bd = measure_betas(m, [1.0, 2.0, 3.0], 20, warmup=5, sweeps=10, caching=False, mode="dqmc")
    assert bu.shape == (3, 4, 4)
