"""The allocation-free entry point lqmc_sweep_static against the handle-based engine.

lqmc_sweep_static serves callers that cannot call cudaMalloc themselves or through the
library: applications whose device memory belongs to their own allocator, and time-stepping
loops that cannot afford the device-wide synchronisation of cudaMalloc/cudaFree.  The
caller passes device buffers it owns; the sweep's scratch lives in a static device array
inside the library.  This test owns its buffers through torch (the test is the caller),
runs two calls in a row, and checks each call's results against the same chain swept by
the existing entry point (lqmc_sweep through Engine).  This file is collected last.
"""
import ctypes

import numpy as np
import pytest
from scipy.linalg import expm

from latticeqmc_gb300 import ChainSpec, Engine, HubbardModel, _native
from latticeqmc_gb300.engine import exp_constants

pytestmark = pytest.mark.gpu


class StaticChain(ctypes.Structure):
    _fields_ = [("n_sites", ctypes.c_int32), ("n_slices", ctypes.c_int32),
                ("stab_every", ctypes.c_int32), ("rng", ctypes.c_int32),
                ("seed", ctypes.c_uint64), ("chain_id", ctypes.c_int32),
                ("measure", ctypes.c_int32), ("exp_consts", ctypes.c_double * 4),
                ("u", ctypes.c_double),
                ("exp_k", ctypes.c_void_p), ("exp_k_t", ctypes.c_void_p),
                ("exp_k_inv", ctypes.c_void_p), ("exp_k_inv_t", ctypes.c_void_p),
                ("kinetic", ctypes.c_void_p), ("field", ctypes.c_void_p),
                ("uniforms", ctypes.c_void_p), ("green", ctypes.c_void_p),
                ("green_sum", ctypes.c_void_p), ("obs", ctypes.c_void_p),
                ("diag", ctypes.c_void_p), ("status", ctypes.c_void_p),
                ("error_message", ctypes.c_char_p), ("error_capacity", ctypes.c_size_t)]


def _dev(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).cuda()


def _static_case(side, L, stab, replay, seed=11):
    """Two lqmc_sweep_static calls of two sweeps each on buffers the test owns, each checked
    against the same chain swept by Engine (lqmc_sweep) from the same inputs."""
    torch = pytest.importorskip("torch")
    lib = _native.load()
    U, beta = 4.0, 2.0
    m = HubbardModel(u=U, t=1, mu=0)
    m.build_square(side)
    K = m.ham_kinetic()
    N = side * side
    rng = np.random.default_rng(seed)
    field = (2 * rng.integers(0, 2, (N, L)) - 1).astype(np.int8)
    spec = ChainSpec(K, U, beta, L, field)
    eki = expm(spec.dtau * K)
    eng = Engine([spec], mode="dqmc", rng="replay" if replay else "philox", seed=seed,
                 stab_every=stab)

    # the caller's own device buffers (allocated here, by the caller, not by the library)
    bufs = {
        "exp_k": _dev(torch, spec.exp_k, torch.float64),
        "exp_k_t": _dev(torch, spec.exp_k.T, torch.float64),
        "exp_k_inv": _dev(torch, eki, torch.float64),
        "exp_k_inv_t": _dev(torch, eki.T, torch.float64),
        "kinetic": _dev(torch, K, torch.float64),
        "field": _dev(torch, field.T, torch.int8),          # [slice][site]
        "green": torch.zeros(2 * N * N, dtype=torch.float64, device="cuda"),
        "green_sum": torch.zeros(2 * N * N, dtype=torch.float64, device="cuda"),
        "obs": torch.zeros(_native.obs_len(N), dtype=torch.float64, device="cuda"),
        "diag": torch.zeros(_native.DIAG_LEN, dtype=torch.float64, device="cuda"),
        "status": torch.zeros(1, dtype=torch.int32, device="cuda"),
    }
    err = ctypes.create_string_buffer(256)
    sc = StaticChain(n_sites=N, n_slices=L, stab_every=stab, rng=0 if replay else 1, seed=seed,
                     chain_id=0, measure=1, u=U, uniforms=None,
                     error_message=ctypes.cast(err, ctypes.c_char_p), error_capacity=256)
    sc.exp_consts[:] = list(exp_constants(spec.lamb, N))
    for k, t in bufs.items():
        setattr(sc, k, t.data_ptr())

    try:
        for call in range(2):
            if replay:
                u = rng.random(2 * N * L)
                u_dev = _dev(torch, u, torch.float64)   # the caller's uniforms of this call
                sc.uniforms = u_dev.data_ptr()
                eng.set_uniforms(0, u)
            rc = lib.lqmc_sweep_static(ctypes.byref(sc), 2, None)
            assert rc == 0, err.value
            torch.cuda.synchronize()
            eng.sweep(2, measure=True)
            g_ref = eng.green(0)
            gs_ref, cnt = eng.green_sum(0)
            g = bufs["green"].cpu().numpy().reshape(2, N, N)
            gs = bufs["green_sum"].cpu().numpy().reshape(2, N, N)
            assert np.abs(g - g_ref).max() < 1e-10, f"call {call}"
            assert np.abs(gs - gs_ref).max() < 1e-10, f"call {call}"
            np.testing.assert_array_equal(bufs["field"].cpu().numpy().T, eng.field(0))
            np.testing.assert_allclose(bufs["obs"].cpu().numpy(), eng.observables_raw(0), atol=1e-10)
            d = bufs["diag"].cpu().numpy()
            assert d[7] == 2 * (call + 1) and cnt == 2 * (call + 1)
            assert int(bufs["status"].cpu().item()) == 0
    finally:
        eng.close()


def test_static_sweep_matches_engine_on_two_calls():
    _static_case(4, 20, 5, replay=False)


def test_static_sweep_replays_the_callers_uniforms_on_two_calls():
    """LQMC_RNG_REPLAY: each call draws from the uniforms buffer the caller passes."""
    _static_case(4, 20, 5, replay=True, seed=12)


def test_static_sweep_at_the_largest_lattice_with_two_chunks():
    """n_sites = LQMC_STATIC_MAX_SITES (8 x 8) with L = 2 stab_every: two chunks of slices,
    the right-product stack of the scratch array in use."""
    _static_case(8, 20, 10, replay=False, seed=13)


def test_static_sweep_rejects_sizes_beyond_its_array():
    lib = _native.load()
    err = ctypes.create_string_buffer(256)
    sc = StaticChain(n_sites=65, n_slices=10, stab_every=5, rng=1,
                     error_message=ctypes.cast(err, ctypes.c_char_p), error_capacity=256)
    assert lib.lqmc_sweep_static(ctypes.byref(sc), 1, None) == -1
    assert b"n_sites <= 64" in err.value
    sc = StaticChain(n_sites=64, n_slices=400, stab_every=1, rng=1,
                     error_message=ctypes.cast(err, ctypes.c_char_p), error_capacity=256)
    for name in ("exp_k", "exp_k_t", "exp_k_inv", "exp_k_inv_t", "kinetic", "field", "green",
                 "green_sum", "obs", "diag", "status"):
        setattr(sc, name, 256)   # never dereferenced: the size check rejects first
    assert lib.lqmc_sweep_static(ctypes.byref(sc), 1, None) == -1
    assert b"static array holds" in err.value
