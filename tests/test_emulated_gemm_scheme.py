"""The digit scheme of the emulated float64 GEMM (latticeqmc_gb300/csrc/ozaki_tc.cuh), restated
in NumPy integers and checked on the CPU against exact rational products.

Scheme as the kernel runs it:

- Each row of A (column of B) gets the exponent E with |x| < 2^E over the row.
- Each entry becomes N = round(x 2^(55 - E)), so |N| <= 2^55.
- N is written as 8 balanced base-128 digits q_t in [-64, 64]. The digits are the 7-bit
  fields of N + 64 (2^56 - 1) / 127, minus 64; the top field is 8 bits wide.
- The 36 digit pairs with t + u <= 7 are summed into 8 diagonals D_d. On the GPU these are
  BF16 products with exact FP32 accumulation.
- The diagonals are combined by Horner in int64 with the 12 low bits dropped, then scaled
  back by 2^(E_i + F_j - 110 + 49 + 12).

These tests pin the scheme's arithmetic (exact digit decomposition, error bound) independently
of the GPU; the GPU kernels are checked against the oracle chain in test_gpu_tiled.py.
"""
from fractions import Fraction

import numpy as np
import pytest

BITS, SLICES, WIDTH = 7, 8, 55
BIAS = 0x81020408102040          # 64 in every base-128 digit


def row_exponents(x):
    """E_r with |x[r, :]| < 2^E_r (0 for an all-zero row), as split_tiles' exps."""
    m = np.abs(x).max(axis=1)
    _, e = np.frexp(m)                      # m = f 2^e, f in [0.5, 1): m < 2^e
    return np.where(m > 0, e, 0).astype(np.int64)


def fixed55(x, e):
    """N = round(x 2^(55 - E)) per row, ties away from zero (fixed55)."""
    n = np.empty(x.shape, dtype=np.int64)
    for r in range(x.shape[0]):
        for q in range(x.shape[1]):
            v = Fraction(float(x[r, q])) * Fraction(2) ** (WIDTH - int(e[r]))
            a = abs(v)
            mag = int(a + Fraction(1, 2))   # floor(|v| + 1/2): ties away from zero
            n[r, q] = mag if v >= 0 else -mag
    return n


def digits(n):
    """Balanced base-128 digits q_t (t = 0 most significant) of N, shape (8,) + N.shape."""
    m = n.astype(np.int64) + BIAS
    out = []
    for t in range(SLICES):
        sh = BITS * (SLICES - 1 - t)
        mask = 0xFF if t == 0 else 0x7F
        out.append(((m >> sh) & mask) - 64)
    return np.stack(out)


def emulated_product(a, b, round_low=False):
    """C = A B through the digit scheme: A (m x k) split by rows, B (k x n) by columns.
    round_low: round the 12 dropped low bits to nearest (LQMC_OZ_ROUND_EPILOGUE=1) instead
    of flooring them."""
    ea, eb = row_exponents(a), row_exponents(b.T)
    qa, qb = digits(fixed55(a, ea)), digits(fixed55(b.T, eb))      # (8, m, k), (8, n, k)
    d = np.zeros((SLICES,) + (a.shape[0], b.shape[1]), dtype=np.int64)
    for t in range(SLICES):
        for u in range(SLICES - t):
            d[t + u] += qa[t] @ qb[u].T
    hi = np.zeros(d.shape[1:], dtype=np.int64)
    lo = np.zeros(d.shape[1:], dtype=np.int64)
    for k in range(SLICES // 2):
        hi = hi * (1 << BITS) + d[k]
        lo = lo * (1 << BITS) + d[SLICES // 2 + k]
    t_int = hi * (1 << (BITS * SLICES // 2 - 12)) + ((lo + (2048 if round_low else 0)) >> 12)
    scale = ea[:, None] + eb[None, :] - 2 * WIDTH + BITS * (SLICES - 1) + 12
    return np.ldexp(t_int.astype(np.float64), scale), ea, eb, d


def exact_product(a, b):
    fa = [[Fraction(float(v)) for v in row] for row in a]
    fb = [[Fraction(float(v)) for v in row] for row in b]
    return [[sum(fa[i][p] * fb[p][j] for p in range(a.shape[1])) for j in range(b.shape[1])]
            for i in range(a.shape[0])]


def graded(rng, shape, span):
    """Entries of random sign and magnitude, rows scaled by 2^(-span .. span)."""
    x = rng.standard_normal(shape) * np.exp(rng.uniform(-3, 3, shape))
    return x * np.ldexp(1.0, rng.integers(-span, span + 1, (shape[0], 1)))


def test_digits_are_balanced_and_exact():
    rng = np.random.default_rng(1)
    x = graded(rng, (16, 24), 40)
    x[3, 5] = 0.0
    x[7, :] = 0.0
    e = row_exponents(x)
    n = fixed55(x, e)
    assert np.abs(n).max() <= 2 ** WIDTH
    q = digits(n)
    assert q.min() >= -64 and q.max() <= 64
    recon = sum(q[t].astype(object) * (1 << (BITS * (SLICES - 1 - t))) for t in range(SLICES))
    assert (recon == n.astype(object)).all()
    # 56 significant bits: the rounding of each entry is at most 2^-56 of its row's scale
    err = np.abs(np.ldexp(n.astype(np.float64), (e - WIDTH)[:, None]) - x)
    assert (err <= np.ldexp(1.0, e - 56)[:, None] * (1 + 1e-12)).all()


def test_extreme_entries_split_without_overflow():
    # entries at the row's maximum give |N| = 2^55 - 4: the 8-bit top field holds q_0 = +-64
    # and the carry-free extraction still reconstructs them; far smaller entries round to 0
    x = np.array([[np.nextafter(1.0, 0.0), -np.nextafter(1.0, 0.0), 0.5, -0.25, 2.0 ** -60]])
    n = fixed55(x, row_exponents(x))
    assert list(n[0]) == [2 ** 55 - 4, -(2 ** 55 - 4), 2 ** 54, -(2 ** 53), 0]
    q = digits(n)
    assert list(q[:, 0, 0]) == [64, 0, 0, 0, 0, 0, 0, -4]
    assert list(q[:, 0, 1]) == [-64, 0, 0, 0, 0, 0, 0, 4]
    for c in range(x.shape[1]):
        assert sum(int(q[t, 0, c]) << (BITS * (SLICES - 1 - t)) for t in range(SLICES)) == int(n[0, c])


@pytest.mark.parametrize("m,k,n,span", [(8, 16, 8, 0), (12, 40, 10, 30), (5, 64, 7, 200)])
def test_product_within_float64_error_bound(m, k, n, span):
    rng = np.random.default_rng(m * k + n)
    a = graded(rng, (m, k), span)
    b = graded(rng, (n, k), span).T.copy()
    c, ea, eb, d = emulated_product(a, b)
    # the diagonal sums stay exact FP32 integers on the tensor cores: |D_d| <= 8 k 64^2
    assert np.abs(d).max() <= 8 * k * 64 * 64 < 2 ** 24
    ex = exact_product(a, b)
    # bound per entry, in units of 2^(E_i + F_j): operand rounding 2 k 2^-56, dropped digit
    # pairs (t + u >= 8) k 7 2^-56, the 12 dropped low bits 2^-48, the final rounding 2^-53
    # of |C| <= k 2^(E_i + F_j)
    bound_units = k * (2 + 7) * 2.0 ** -56 + 2.0 ** -48 + k * 2.0 ** -53
    plain = a @ b
    worst, worst_plain = 0.0, 0.0
    for i in range(m):
        for j in range(n):
            unit = 2.0 ** (int(ea[i]) + int(eb[j]))
            err = abs(Fraction(float(c[i, j])) - ex[i][j])
            assert err <= Fraction(bound_units) * Fraction(unit), (i, j)
            worst = max(worst, float(err) / (k * unit))
            worst_plain = max(worst_plain, float(abs(Fraction(float(plain[i, j])) - ex[i][j])) / (k * unit))
    # observed: within 2^-49 (the floored low bits, below) + a few units of 2^-56 per term
    assert worst * k <= 2.0 ** -49 + k * 4 * 2.0 ** -56, (worst, worst_plain)


@pytest.mark.parametrize("round_low", [False, True])
def test_epilogue_drop_of_low_bits(round_low):
    """The combine floors the 12 low bits of sum_d D_d 2^(7 (7 - d)) (lo >> 12): against the
    same diagonals combined exactly, every product moves down by less than 2^-49 2^(E_i + F_j)
    (plus the final float64 rounding), whatever k is.  At small k this term dominates the
    error, and it is a bias rather than noise.  Rounding instead (LQMC_OZ_ROUND_EPILOGUE=1)
    bounds the move by 2^-50 of 2^(E_i + F_j) in either direction and removes the bias."""
    rng = np.random.default_rng(7)
    for k in (4, 64):
        a = graded(rng, (12, k), 0)
        b = graded(rng, (12, k), 0).T.copy()
        c, ea, eb, d = emulated_product(a, b, round_low)
        shifts = []
        for i in range(12):
            for j in range(12):
                x = sum(int(d[dd, i, j]) << (BITS * (SLICES - 1 - dd)) for dd in range(SLICES))
                unit = Fraction(2) ** (int(ea[i]) + int(eb[j]))
                combined = Fraction(x) * Fraction(2) ** (BITS * (SLICES - 1) - 2 * WIDTH) * unit
                shift = (Fraction(float(c[i, j])) - combined) / unit
                fl = abs(combined / unit) * Fraction(2) ** -53     # the final float64 rounding
                lo, hi = (-Fraction(2) ** -50, Fraction(2) ** -50) if round_low else (-Fraction(2) ** -49, 0)
                assert lo - fl <= shift <= hi + fl
                shifts.append(float(shift))
        if round_low:
            assert abs(np.mean(shifts)) < 2.0 ** -53     # no bias
        else:
            assert np.mean(shifts) < -2.0 ** -52         # one-signed: a bias of ~2^-50
