"""Generate ``compat_8x8_long.npz``: the reference's fast-sweep decision stream for 500 sweeps
of the 8x8, beta=4, L=80 chain (U=4, mu=0) that ``compat_8x8.npz`` recorded for 2 sweeps.

The reference takes ~15 s per sweep here (its pure-Python rank-1 loop), so the 500 sweeps are
restated by ``oracle/compat.py`` with ``rank1='outer'``, which is bit-identical to the
reference on every recorded sweep (tests/test_oracle.py).  Inputs come from
``compat_8x8.npz`` (exp_k, lambda, the initial field): numpy's legacy generator seeded with
the fixture's seed draws the field as ``Configuration.initialize`` does
(lqmc/configuration.py:120-124) and then one ``np.random.rand()`` per site in sweep order
(lqmc/lqmc.py:313-317); the test regenerates that stream from the seed.

Stored: the decisions of every sweep (packed bits), the flat indices of "near ties" -- sites
where |u - ratio| < NEAR_TIE, at which a float64 restatement with another summation order
may decide the other way (the reference's unstabilised wraps amplify rounding to ~1e-5 in G
on 8x8) -- and the final field.

    python tests/golden/make_compat_long.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import compat  # noqa: E402

N_SWEEPS = 500
NEAR_TIE = 1e-3


def main():
    f = np.load(os.path.join(HERE, "compat_8x8.npz"))
    n, L = f["field0"].shape
    np.random.seed(int(f["seed"]))
    field = (2 * np.random.randint(0, 2, size=(n, L)) - 1).astype(np.int8)
    assert np.array_equal(field, f["field0"])
    uni = np.random.rand(N_SWEEPS * n * L)
    assert np.array_equal(uni[:f["uniforms"].size], f["uniforms"])
    acc = np.zeros((N_SWEEPS, L, n), np.int8)
    near = []
    for sw in range(N_SWEEPS):
        u = uni[sw * n * L:(sw + 1) * n * L]
        rec = {}
        compat.update_step(f["exp_k"], field, float(f["lamb"]), u, record=rec)
        acc[sw] = rec["accept"]
        close = np.nonzero(np.abs(u - rec["ratio"].ravel()) < NEAR_TIE)[0]
        near.append(close + sw * n * L)
        if sw < f["accept"].shape[0]:
            assert np.array_equal(rec["accept"], f["accept"][sw])
    np.savez_compressed(os.path.join(HERE, "compat_8x8_long.npz"), seed=int(f["seed"]),
                        n_sweeps=N_SWEEPS, near_tie=NEAR_TIE,
                        accept_bits=np.packbits(acc.ravel()),
                        near_idx=np.concatenate(near).astype(np.int32), field_end=field)
    print(f"{N_SWEEPS} sweeps, acceptance {acc.mean():.3f}, near ties "
          f"{sum(len(x) for x in near)}")


if __name__ == "__main__":
    main()
