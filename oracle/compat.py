"""Oracle: numpy restatement of the reference fast sweep (TEST INFRASTRUCTURE ONLY).

This is the checker for the engine's ``compat`` mode.  It restates, operation for
operation, the arithmetic of KieDani/LatticeQMC ``lqmc/lqmc.py``:

* ``set_beta``        lqmc.py:93-117   (lambda = arccosh(exp(U dtau/2)), exp_k = expm(-dtau K))
* ``get_exp_v``       lqmc.py:132-154  (diag(exp(-sigma lambda s[:, l])))
* ``get_m``           lqmc.py:156-185  (M = 1 + prod_{l=L-1..0} exp_k . exp_v(l))
* ``_update_step``    lqmc.py:301-347  (ratio, Sherman-Morrison update, wrap)

including the reference's defects (the ratio reads a G whose leftmost factor is exp_k,
the update uses the opposite spin's Delta, the wrap goes the "upward" way, and nothing is
stabilised).  Every floating-point operation is the same numpy call form as in the
reference, so on the same numpy/BLAS build the results are bit-identical; the tests pin
that against the fixtures recorded from the reference (tests/golden/compat_*.npz).

The pure-Python ``j, k`` double loop of lqmc.py:328-331 is kept as ``rank1='loop'``
(used to time the reference's CPU cost); ``rank1='outer'`` computes the same products
and differences element by element with numpy and is bit-identical.
"""
import numpy as np
from scipy.linalg import expm


def set_beta(kinetic, u, beta, time_steps):
    """lqmc.py:102-106 -> (dtau, lamb, exp_k)."""
    dtau = beta / time_steps
    lamb = np.arccosh(np.exp(u * dtau / 2.)) if u else 0
    exp_k = expm(-1 * dtau * kinetic)
    return dtau, lamb, exp_k


def get_exp_v(field, lamb, l, sigma):
    """lqmc.py:149-154."""
    diag = -1 * sigma * lamb * field[:, l]
    return np.diagflat(np.exp(diag))


def get_m(exp_k, field, lamb, l0, sigma):
    """lqmc.py:173-185: M = 1 + B_{l0} ... B_{l0+1} (cyclic, B = exp_k exp_v)."""
    n_sites, time_steps = field.shape
    l0 = l0 % time_steps
    indices = list(reversed(range(time_steps)))
    time_indices = indices[-l0:] + indices[:-l0]
    b_prod = 1
    for l in time_indices:
        exp_v = get_exp_v(field, lamb, l, sigma)
        b = np.dot(exp_k, exp_v)
        b_prod = np.dot(b_prod, b)
    return np.eye(n_sites) + b_prod


def greens_from_scratch(exp_k, field, lamb):
    """lqmc.py:303-307: the unstabilised recompute at the start of every sweep."""
    gf_up = np.linalg.inv(get_m(exp_k, field, lamb, 0, +1))
    gf_dn = np.linalg.inv(get_m(exp_k, field, lamb, 0, -1))
    return gf_up, gf_dn


class _SampleDone(Exception):
    pass


def update_step(exp_k, field, lamb, uniforms, rank1="outer", record=None, max_sites=None,
                log_line=False):
    """One fast sweep, lqmc.py:301-347.

    Parameters
    ----------
    exp_k : (N, N) float64       expm(-dtau K)
    field : (N, L) int8          Hubbard-Stratonovich field, flipped in place
    lamb : float                 HS coupling
    uniforms : (L*N,) float64    the uniforms in sweep order (l = L-1..0, i = 0..N-1);
                                 the reference draws exactly one np.random.rand() per site
    record : dict or None        if given, receives 'accept' (L, N) int8 and 'ratio' (L, N)
                                 indexed [L-1-l_step, i] in sweep order
    max_sites : int or None      stop after this many site updates and return None (used to
                                 time a bounded sample of a sweep)
    log_line : bool              also build the per-site log line the reference formats on
                                 every site, logger or not (lqmc.py:217-232, :335)

    Returns (gf_up, gf_dn) after slice 0 (not wrapped), as lqmc.py:347.
    """
    n_sites, time_steps = field.shape
    gf_up, gf_dn = greens_from_scratch(exp_k, field, lamb)
    acc_rec = np.zeros((time_steps, n_sites), np.int8)
    rat_rec = np.zeros((time_steps, n_sites))
    pos = 0
    for step, l in enumerate(reversed(range(time_steps))):
        for i in range(n_sites):
            arg = 2 * lamb * field[i, l]
            d_up = 1 + (1 - gf_up[i, i]) * (np.exp(+arg) - 1)
            d_dn = 1 + (1 - gf_dn[i, i]) * (np.exp(-arg) - 1)
            ratio = d_up * d_dn
            acc = uniforms[pos] <= ratio
            pos += 1
            acc_rec[step, i] = acc
            rat_rec[step, i] = ratio
            if max_sites is not None and pos > max_sites:
                raise _SampleDone()
            if acc:
                c_up = -(np.exp(-arg) - 1) * gf_up[i, :]
                c_up[i] += (np.exp(-arg) - 1)
                c_dn = -(np.exp(+arg) - 1) * gf_dn[i, :]
                c_dn[i] += (np.exp(+arg) - 1)
                e_up = gf_up[:, i] / (1 + c_up[i])
                e_dn = gf_dn[:, i] / (1 + c_dn[i])
                if rank1 == "loop":
                    for j in range(n_sites):
                        for k in range(n_sites):
                            gf_up[j, k] = gf_up[j, k] - e_up[j] * c_up[k]
                            gf_dn[j, k] = gf_dn[j, k] - e_dn[j] * c_dn[k]
                else:
                    # elementwise product then difference: one rounding each, as above
                    gf_up = gf_up - e_up[:, None] * c_up[None, :]
                    gf_dn = gf_dn - e_dn[:, None] * c_dn[None, :]
                field[i, l] *= -1
            if log_line:
                _ = f"{l:>2} {i:>2} -- {ratio:.1f} ({acc}) -- {np.mean(field):.3f} {np.var(field):.3f}"
        if l > 0:
            exp_v_up = get_exp_v(field, lamb, l - 1, +1)
            exp_v_dn = get_exp_v(field, lamb, l - 1, -1)
            b_up = np.dot(exp_v_up, exp_k)
            b_dn = np.dot(exp_v_dn, exp_k)
            gf_up = np.dot(np.dot(b_up, gf_up), np.linalg.inv(b_up))
            gf_dn = np.dot(np.dot(b_dn, gf_dn), np.linalg.inv(b_dn))
    if record is not None:
        record["accept"] = acc_rec
        record["ratio"] = rat_rec
    return gf_up, gf_dn


def time_sites(exp_k, field, lamb, uniforms, n_sites_sample):
    """Seconds per site update of the reference's fast sweep (pure-Python rank-1 loop and
    per-site log line, as lqmc.py:301-347 runs with log_lvl=None), timed over the first
    ``n_sites_sample`` site updates of a sweep."""
    import time
    t0 = time.perf_counter()
    try:
        update_step(exp_k, field, lamb, uniforms, rank1="loop", max_sites=n_sites_sample,
                    log_line=True)
        done = field.size
    except _SampleDone:
        done = n_sites_sample
    return (time.perf_counter() - t0) / done


def run(exp_k, field, lamb, uniforms, warmup, sweeps):
    """lqmc.py:349-393 (warmup_loop, measure_loop): mean of end-of-sweep G."""
    n_sites, time_steps = field.shape
    per = n_sites * time_steps
    pos = 0
    for _ in range(warmup):
        update_step(exp_k, field, lamb, uniforms[pos:pos + per])
        pos += per
    tot_up = np.zeros((n_sites, n_sites))
    tot_dn = np.zeros((n_sites, n_sites))
    for _ in range(sweeps):
        gu, gd = update_step(exp_k, field, lamb, uniforms[pos:pos + per])
        pos += per
        tot_up += gu
        tot_dn += gd
    return np.asarray([tot_up, tot_dn]) / sweeps


def exp_constants(lamb, n_sites=64):
    """The four exponentials the compat kernel needs, in the reference's call forms.

    exp(+-2 lamb) come from numpy scalar exp of arg = 2*lamb*s (lqmc.py:313-323);
    exp(-+lamb) come from numpy array exp over a field column (lqmc.py:149-154).
    Returns [exp(2l), exp(-2l), exp(-l), exp(+l)] =
    [exp(arg) for s=+1, exp(arg) for s=-1, exp_v entry for sigma*s=+1, for sigma*s=-1].
    """
    lamb = np.float64(lamb)
    s_pos = np.int8(1)
    s_neg = np.int8(-1)
    e2p = np.exp(+(2 * lamb * s_pos))
    e2m = np.exp(+(2 * lamb * s_neg))
    col = np.array(([1, -1] * ((n_sites + 1) // 2))[:max(n_sites, 2)], dtype=np.int8)
    ev = np.exp(-1 * 1 * lamb * col)
    return np.array([e2p, e2m, ev[0], ev[1]], dtype=np.float64)
