"""The emulated float64 GEMM of the fp64e engine on its own (lqmc_emulated_gemm), against
float64 products: every shape class the sweep uses (square lattice products, delayed-update
flushes with small k, ragged sizes, k beyond one exact chunk), both operand orientations,
operands split up front, the subtract / row-scale / column-scale epilogue, graded rows and
columns, and non-finite propagation.

Bound: each operand row (column) is carried as a 55-bit fixed-point integer relative to a
power of two 2^E just above its largest entry, so |C - AB|_ij <= (2^-50 + k 2^-54) 2^(E_i + F_j)
up to a small factor; numpy's own float64 error is far below that."""
import numpy as np
import pytest

from latticeqmc_gb300 import _native

pytestmark = pytest.mark.gpu


def _bound(a_op, b_op):
    k = a_op.shape[1]
    ra = 2.0 ** np.ceil(np.log2(np.maximum(np.abs(a_op).max(axis=1), 1e-300)))
    cb = 2.0 ** np.ceil(np.log2(np.maximum(np.abs(b_op).max(axis=0), 1e-300)))
    return 4.0 * (2.0 ** -50 + k * 2.0 ** -54) * np.outer(ra, cb)


@pytest.mark.parametrize("m,n,k", [(256, 256, 256), (100, 100, 100), (37, 53, 24), (256, 256, 24),
                                   (64, 96, 1024), (130, 33, 17)])
@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
def test_product_within_the_fixed_point_bound(m, n, k, ta, tb):
    rng = np.random.default_rng(m * 7 + n * 3 + k + 11 * ta + 5 * tb)
    a_op = rng.standard_normal((m, k)) * np.exp(rng.uniform(-3, 3, (m, 1)))
    b_op = rng.standard_normal((k, n)) * np.exp(rng.uniform(-3, 3, (1, n)))
    a = a_op.T.copy() if ta else a_op
    b = b_op.T.copy() if tb else b_op
    c, cyc = _native.emulated_gemm(a, b, trans_a=ta, trans_b=tb)
    err = np.abs(c - a_op @ b_op)
    assert (err <= _bound(a_op, b_op)).all(), f"worst ratio {(err / _bound(a_op, b_op)).max():.2f}"
    assert cyc[1] > 0


@pytest.mark.parametrize("stages", [1, 2, 3])
def test_stage_counts_and_presplit_operands_give_identical_results(stages):
    rng = np.random.default_rng(stages)
    a = rng.standard_normal((256, 256))
    b = rng.standard_normal((256, 256))
    ref, _ = _native.emulated_gemm(a, b, stages=2)
    for pa, pb in ((False, False), (True, False), (False, True)):
        c, _ = _native.emulated_gemm(a, b, stages=stages, presplit_a=pa, presplit_b=pb)
        np.testing.assert_array_equal(c, ref)


def test_subtract_and_scaled_epilogue():
    """C - diag(r) A B diag(s): the delayed-update flush (subtract) and the wrap's / B-chain's
    row and column scalings."""
    rng = np.random.default_rng(3)
    m, n, k = 200, 160, 24
    a = rng.standard_normal((m, k))
    b = rng.standard_normal((n, k))
    c0 = rng.standard_normal((m, n))
    r = np.exp(rng.uniform(-1, 1, m))
    s = np.exp(rng.uniform(-1, 1, n))
    c, _ = _native.emulated_gemm(a, b, c=c0, trans_b=True, subtract=True, row_scale=r, col_scale=s)
    exact = c0 - (r[:, None] * (a @ b.T)) * s[None, :]
    bound = _bound(a, b.T) * np.outer(r, s) * 2 + 4 * np.finfo(float).eps * np.abs(exact)
    assert (np.abs(c - exact) <= bound).all()


def test_graded_operands_keep_relative_row_and_column_accuracy():
    """Rows of A and columns of B spanning 1e-150 .. 1e150: the error of each output stays
    relative to its own row and column scale."""
    rng = np.random.default_rng(4)
    m = n = k = 96
    a = rng.standard_normal((m, k)) * (10.0 ** rng.uniform(-150, 150, (m, 1)))
    b = rng.standard_normal((k, n)) * (10.0 ** rng.uniform(-150, 150, (1, n)))
    c, _ = _native.emulated_gemm(a, b)
    assert (np.abs(c - a @ b) <= _bound(a, b)).all()


def test_nonfinite_rows_and_columns_give_nan():
    rng = np.random.default_rng(5)
    a = rng.standard_normal((40, 30))
    b = rng.standard_normal((30, 50))
    a[7, 3] = np.nan
    b[2, 11] = np.inf
    c, _ = _native.emulated_gemm(a, b)
    assert np.isnan(c[7]).all() and np.isnan(c[:, 11]).all()
    mask = np.ones_like(c, bool)
    mask[7] = False
    mask[:, 11] = False
    assert np.isfinite(c[mask]).all()
