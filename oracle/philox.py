"""Oracle: Philox4x64-10 counter-based generator (TEST INFRASTRUCTURE ONLY).

Restates the published Philox4x64 algorithm (Salmon, Moraes, Dror, Shaw, "Parallel random
numbers: as easy as 1, 2, 3", SC'11): 10 rounds of two 64x64->128-bit multiplies with the
multipliers 0xD2E7470EE14C6C93 / 0xCA5A826395121157 and Weyl key increments
0x9E3779B97F4A7C15 / 0xBB67AE8584CAA73B.  numpy's ``np.random.Philox`` implements the same
function; the tests pin this restatement against it.

The engine's ``philox`` RNG mode draws the uniform of site position ``p`` (sweep order,
p = (L-1-l)*N + i) of sweep ``t`` of chain ``c`` as word ``p % 4`` of
``philox4x64(counter=(p // 4, t, 0, 0), key=(seed, c))``, converted to a double in [0, 1)
as ``(word >> 11) * 2**-53`` (the same conversion numpy uses for ``random()``).
"""
import numpy as np

M0 = 0xD2E7470EE14C6C93
M1 = 0xCA5A826395121157
W0 = 0x9E3779B97F4A7C15
W1 = 0xBB67AE8584CAA73B
MASK = (1 << 64) - 1


def philox4x64(counter, key, rounds=10):
    c0, c1, c2, c3 = (int(x) & MASK for x in counter)
    k0, k1 = (int(x) & MASK for x in key)
    for r in range(rounds):
        if r:
            k0 = (k0 + W0) & MASK
            k1 = (k1 + W1) & MASK
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> 64, p0 & MASK
        hi1, lo1 = p1 >> 64, p1 & MASK
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return [c0, c1, c2, c3]


def uniforms(seed, chain, sweep, n_sites, time_steps):
    """The N*L uniforms of one sweep in sweep order (float64)."""
    n = n_sites * time_steps
    out = np.empty(n, dtype=np.float64)
    for b in range((n + 3) // 4):
        words = philox4x64((b, sweep, 0, 0), (seed, chain))
        for w in range(4):
            p = 4 * b + w
            if p < n:
                out[p] = (words[w] >> 11) * (1.0 / 9007199254740992.0)
    return out
