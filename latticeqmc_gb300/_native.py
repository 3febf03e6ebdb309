"""ctypes binding of liblqmc_gpu.so (the C ABI in include/lqmc_gpu.h).

The library is built in-tree by ``latticeqmc_gb300.build``.  There is no CPU fallback:
if the library is missing or no CUDA device is present, loading or ``lqmc_create`` fails
with an exception.
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "liblqmc_gpu.so")

LQMC_OK = 0
ERRORS = {-1: "LQMC_ERR_INVALID", -2: "LQMC_ERR_CUDA", -3: "LQMC_ERR_STATE",
          -4: "LQMC_ERR_UNSUPPORTED", -5: "LQMC_ERR_NUMERIC", -6: "LQMC_ERR_NOMEM"}
MODES = {"compat": 0, "dqmc": 1, "det": 2}
PRECISIONS = {"fp64": 0, "mixed": 1, "fp64e": 2}
RNGS = {"replay": 0, "philox": 1}
ENGINES = {"auto": 0, "smem": 1, "tiled": 2}
ORDERS = {"down": 0, "alternate": 1}
STATUS_NONFINITE, STATUS_SINGULAR, STATUS_DRIFT, STATUS_TIMEOUT = 1, 2, 4, 8
DEBUG_STALL_TC_WAIT = 1
GEMM_SUBTRACT, GEMM_KSCALE, GEMM_PRESPLIT_A, GEMM_PRESPLIT_B = 1, 2, 4, 8
FP64E_NATIVE = {"wrap": 1, "stack": 2, "udt": 4, "green": 8, "update": 16, "lu": 32,
                "lu_rhs": 64}
OBS_HEADER = 8
DIAG_LEN = 24


def obs_len(n):
    return OBS_HEADER + 2 * n + 2 * n * n


class Params(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("precision", ctypes.c_int32), ("rng", ctypes.c_int32),
                ("stab_every", ctypes.c_int32), ("delay", ctypes.c_int32), ("record", ctypes.c_int32),
                ("seed", ctypes.c_uint64), ("device", ctypes.c_int32), ("engine", ctypes.c_int32),
                ("debug", ctypes.c_int32), ("fp64e_native", ctypes.c_int32),
                ("measure_tau", ctypes.c_int32), ("sweep_order", ctypes.c_int32),
                ("oz_stages", ctypes.c_int32), ("reserved", ctypes.c_int32 * 1)]


class LqmcError(RuntimeError):
    """A negative return code from liblqmc_gpu.so."""

    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


# (name, restype, argtypes) of every exported symbol
_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_SIGS = [
    ("lqmc_abi_version", ctypes.c_int, []),
    ("lqmc_create", ctypes.c_int, [ctypes.POINTER(Params), ctypes.POINTER(_P)]),
    ("lqmc_set_chains", ctypes.c_int, [_P, _I32, _P, _P, _P, _P, _P, _P, _P]),
    ("lqmc_set_field", ctypes.c_int, [_P, _I32, _P]),
    ("lqmc_get_field", ctypes.c_int, [_P, _I32, _P]),
    ("lqmc_set_uniforms", ctypes.c_int, [_P, _I32, _P, ctypes.c_size_t]),
    ("lqmc_set_uniforms_all", ctypes.c_int, [_P, _P, ctypes.c_size_t]),
    ("lqmc_sweep", ctypes.c_int, [_P, _I32, _I32, _P]),
    ("lqmc_get_green", ctypes.c_int, [_P, _I32, _P]),
    ("lqmc_get_green_all", ctypes.c_int, [_P, _P]),
    ("lqmc_get_green_sum", ctypes.c_int, [_P, _I32, _P, _P]),
    ("lqmc_get_observables", ctypes.c_int, [_P, _I32, _P]),
    ("lqmc_reset_measurements", ctypes.c_int, [_P]),
    ("lqmc_get_decisions", ctypes.c_int, [_P, _I32, _P, ctypes.c_size_t]),
    ("lqmc_get_diagnostics", ctypes.c_int, [_P, _I32, _P]),
    ("lqmc_set_chain_state", ctypes.c_int, [_P, _I32, _P, _P, _P]),
    ("lqmc_get_green_tau", ctypes.c_int, [_P, _I32, _P]),
    ("lqmc_set_green_tau", ctypes.c_int, [_P, _I32, _P]),
    ("lqmc_get_status", ctypes.c_int, [_P, _P]),
    ("lqmc_get_launch_count", ctypes.c_int, [_P, _P]),
    ("lqmc_last_error", ctypes.c_char_p, [_P]),
    ("lqmc_destroy", None, [_P]),
    ("lqmc_sweep_static", ctypes.c_int, [_P, _I32, _P]),
    ("lqmc_emulated_gemm", ctypes.c_int, [_I32, _I32, _I32, _P, _I32, _I32, _P, _I32, _I32, _P,
                                          _I32, _P, _P, _I32, _I32, _I32, _P]),
]
EXPORTED = [s[0] for s in _SIGS]

_lib = None


def load():
    """Load liblqmc_gpu.so once; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                               "`python -m latticeqmc_gb300.build` (no CPU fallback exists)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, res, args in _SIGS:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _choice(table, value, what):
    """table[value], or ValueError naming the accepted values (the reference raises ValueError
    for bad arguments, lqmc/multiprocessing.py:108)."""
    try:
        return table[value]
    except (KeyError, TypeError):
        raise ValueError(f"unknown {what} {value!r}; expected one of {sorted(table)}") from None


class Handle:
    """Owns one lqmc_handle; every call checks the return code."""

    def __init__(self, mode, precision, rng, stab_every, delay, seed, record, device,
                 engine="auto", debug=0, fp64e_native=("lu", "lu_rhs"), measure_tau=False,
                 sweep_order="down", oz_stages=0):
        self.lib = load()
        if isinstance(fp64e_native, int):
            native = fp64e_native
        else:
            native = 0
            for name in fp64e_native:
                if name not in FP64E_NATIVE:
                    raise ValueError(f"unknown fp64e product category {name!r}")
                native |= FP64E_NATIVE[name]
        p = Params(mode=_choice(MODES, mode, "mode"),
                   precision=_choice(PRECISIONS, precision, "precision"),
                   rng=_choice(RNGS, rng, "rng"),
                   stab_every=int(stab_every), delay=int(delay), record=int(bool(record)),
                   seed=int(seed) & ((1 << 64) - 1), device=int(device),
                   engine=_choice(ENGINES, engine, "engine"),
                   debug=int(debug), fp64e_native=int(native),
                   measure_tau=int(bool(measure_tau)),
                   sweep_order=_choice(ORDERS, sweep_order, "sweep order"),
                   oz_stages=int(oz_stages))
        h = ctypes.c_void_p()
        rc = self.lib.lqmc_create(ctypes.byref(p), ctypes.byref(h))
        if rc != LQMC_OK:
            raise LqmcError(rc, self.lib.lqmc_last_error(None).decode())
        self.h = h

    def check(self, rc):
        if rc != LQMC_OK:
            raise LqmcError(rc, self.lib.lqmc_last_error(self.h).decode())

    def call(self, name, *args):
        self.check(getattr(self.lib, name)(self.h, *args))

    def close(self):
        if getattr(self, "h", None):
            self.lib.lqmc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def emulated_gemm(a, b, c=None, trans_a=False, trans_b=False, subtract=False, row_scale=None,
                  col_scale=None, kscale=False, presplit_a=False, presplit_b=False, stages=2,
                  device=0):
    """C = op(A) op(B) (or C - op(A) op(B)) through the fp64e engine's emulated float64 GEMM
    on the tensor cores (lqmc_emulated_gemm).  a, b: 2-D float64 arrays as stored (op = the
    transpose when trans_*).  Returns (C, cycles of split / pipeline / drain)."""
    lib = load()
    a = as_f64(a)
    b = as_f64(b)
    m = a.shape[1] if trans_a else a.shape[0]
    k = a.shape[0] if trans_a else a.shape[1]
    n = b.shape[0] if trans_b else b.shape[1]
    if (b.shape[1] if trans_b else b.shape[0]) != k:
        raise ValueError("inner dimensions differ")
    c = np.zeros((m, n)) if c is None else as_f64(c).copy()
    rs = None if row_scale is None else as_f64(row_scale)
    cs = None if col_scale is None else as_f64(col_scale)
    cyc = np.zeros(3)
    flags = ((GEMM_SUBTRACT if subtract else 0) | (GEMM_KSCALE if kscale else 0) |
             (GEMM_PRESPLIT_A if presplit_a else 0) | (GEMM_PRESPLIT_B if presplit_b else 0))
    rc = lib.lqmc_emulated_gemm(m, n, k, ptr(a), a.shape[1], int(trans_a), ptr(b), b.shape[1],
                                int(trans_b), ptr(c), n, None if rs is None else ptr(rs),
                                None if cs is None else ptr(cs), flags, int(stages), int(device),
                                ptr(cyc))
    if rc != LQMC_OK:
        raise LqmcError(rc, "lqmc_emulated_gemm failed")
    return c, cyc
