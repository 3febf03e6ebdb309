"""Oracle: textbook FP64 determinant QMC, numpy (TEST INFRASTRUCTURE ONLY).

This is the checker for the engine's ``dqmc`` mode.  It keeps the reference's model,
field and sweep order (lqmc/lqmc.py:301-347: l = L-1..0, i = 0..N-1, one uniform per site,
accept if ``u <= ratio``, G recomputed from scratch at the start of every sweep) and its
factor conventions (``exp_v = diag(exp(-sigma lambda s))``, lqmc.py:149-154), but with the
three arithmetic defects of the reference's fast path fixed and with stabilisation:

* the ratio reads G~_l = (1 + B_l B_{l-1} ... B_0 B_{L-1} ... B_{l+1})^-1 with
  B_l = exp_v(l) exp_k, i.e. the field factor leftmost; it then equals the reference's
  determinant ratio new_det/old_det (lqmc.py:244-248) to rounding;
* the Sherman-Morrison update uses the flipped spin's own Delta:
  G' = G - (Delta/R) G[:, i] (e_i - G[i, :]),  R = 1 + Delta (1 - G_ii),
  Delta_sigma = exp(2 sigma lambda s_il) - 1;
* the wrap goes down: G~_{l-1} = B_l^-1 G~_l B_l = exp(+dtau K) exp_v(l)^-1 G exp_v(l) exp_k;
* the from-scratch G is a pre-pivoted QR (UDT) chain product (Bai, Lee, Li, Xu, "Stable
  solutions of linear systems involving long chain of matrix multiplications", 2011),
  refreshed every ``stab_every`` slices from a right stack (slices below, built at the
  start of the sweep) and a progressively built left product (slices above, updated).

Measurements (Wick's theorem on the end-of-sweep G~_0) are defined in ``measure``.
"""
import numpy as np


def exp_v_diag(field_col, lamb, sigma):
    return np.exp(-sigma * lamb * field_col.astype(np.float64))


def chunks(time_steps, stab_every):
    n = (time_steps + stab_every - 1) // stab_every
    return [(c * stab_every, min((c + 1) * stab_every, time_steps)) for c in range(n)]


def householder_qr(z):
    """Householder QR, LAPACK sign convention (beta = -sign(alpha) ||x||).

    Returns (q, r, det_q_sign)."""
    z = np.array(z, dtype=np.float64)
    n = z.shape[0]
    q = np.eye(n)
    vs = []
    nrefl = 0
    for j in range(n - 1):
        x = z[j:, j]
        alpha = x[0]
        xnorm = np.sqrt(np.dot(x[1:], x[1:]))
        if xnorm == 0.0:
            vs.append(None)
            continue
        beta = -np.copysign(np.hypot(alpha, xnorm), alpha)
        tau = (beta - alpha) / beta
        v = x / (alpha - beta)
        v[0] = 1.0
        w = tau * (v @ z[j:, j:])
        z[j:, j:] -= np.outer(v, w)
        z[j + 1:, j] = 0.0
        vs.append((v, tau))
        nrefl += 1
    for j in reversed(range(n - 1)):
        if vs[j] is None:
            continue
        v, tau = vs[j]
        w = tau * (v @ q[j:, j:])
        q[j:, j:] -= np.outer(v, w)
    return q, np.triu(z), (-1.0) ** nrefl


def lapack_qr(z):
    """The same Householder QR through LAPACK (numpy.linalg.qr: dgeqrf/dorgqr, whose
    reflectors follow the same beta = -sign(alpha) ||x|| convention), for large matrices
    where the Python loop of householder_qr is slow.  Returns (q, r, det_q_sign)."""
    q, r = np.linalg.qr(z)
    return q, r, float(np.linalg.slogdet(q)[0])


def udt_step(z_times_u, d, t, qr=householder_qr):
    """Absorb a left factor: given Z = C U (U of the old decomposition), return the UDT of
    C U diag(d) T with pre-pivoting by column norms of Z diag(d)."""
    zd = z_times_u * d[None, :]
    norms = np.sqrt(np.sum(zd * zd, axis=0))
    order = np.argsort(-norms, kind="stable")
    q, r, sq = qr(zd[:, order])
    dn = np.diag(r).copy()
    tn = (r / dn[:, None]) @ t[order, :]
    return q, dn, tn, sq


def green_from_udt(right, left):
    """G = (1 + U_R D_R T_R T_L^T D_L U_L^T)^-1 and (log|det G|, sign det G)."""
    ur, dr, tr, sr = right
    ul, dl, tl, sl = left
    dbr = np.maximum(np.abs(dr), 1.0)
    dsr = dr / dbr
    dbl = np.maximum(np.abs(dl), 1.0)
    dsl = dl / dbl
    x = ur.T @ ul
    y = tr @ tl.T
    w = x / dbr[:, None] / dbl[None, :] + dsr[:, None] * y * dsl[None, :]
    rhs = ur.T / dbr[:, None]
    z = np.linalg.solve(w, rhs)
    z = z / dbl[:, None]
    g = ul @ z
    sw, lw = np.linalg.slogdet(w)
    logdet = -(np.sum(np.log(dbr)) + lw + np.sum(np.log(dbl)))
    return g, logdet, sr * sw * sl


def identity_udt(n):
    return (np.eye(n), np.ones(n), np.eye(n), 1.0)


class Chain:
    """One Markov chain of the textbook DQMC (both spins)."""

    def __init__(self, exp_k, exp_k_inv, lamb, field, stab_every, kinetic=None, u=0.0,
                 delay=0, qr="householder"):
        self.exp_k = np.asarray(exp_k, dtype=np.float64)
        self.exp_k_inv = np.asarray(exp_k_inv, dtype=np.float64)
        self.lamb = float(lamb)
        self.field = np.array(field, dtype=np.int8)          # (N, L), reference layout
        self.n, self.L = self.field.shape
        self.stab_every = int(stab_every)
        self.kinetic = kinetic
        self.u = u
        self.green = None
        self.max_resid = 0.0
        self.logdet = np.zeros(2)
        self.sign = np.ones(2)
        # delay > 0: the accepted flips of a slice are applied as delayed rank-k updates
        # (G_eff = G - X Y^T, flushed every `delay` flips and at the end of each slice),
        # the same algebra as the rank-1 update in another order of operations; qr =
        # "lapack" factors the UDT steps through LAPACK.  Both only make large lattices
        # fast enough to check; the defaults are the pinned restatement.
        self.delay = int(delay)
        self.qr = lapack_qr if qr == "lapack" else householder_qr

    def b_left(self, l, sigma, z):
        """B_l z = exp_v(l) exp_k z."""
        return exp_v_diag(self.field[:, l], self.lamb, sigma)[:, None] * (self.exp_k @ z)

    def bt_left(self, l, sigma, z):
        """B_l^T z = exp_k^T exp_v(l) z."""
        return self.exp_k.T @ (exp_v_diag(self.field[:, l], self.lamb, sigma)[:, None] * z)

    def right_stack(self, sigma):
        n = self.n
        u, d, t, s = identity_udt(n)
        stack = []
        for lo, hi in chunks(self.L, self.stab_every):
            z = u
            for l in range(lo, hi):
                z = self.b_left(l, sigma, z)
            u, d, t, sq = udt_step(z, d, t, self.qr)
            s = sq
            stack.append((u, d, t, s))
        return stack

    def left_step(self, sigma, left, lo, hi):
        u, d, t, _ = left
        z = u
        for l in reversed(range(lo, hi)):
            z = self.bt_left(l, sigma, z)
        u, d, t, sq = udt_step(z, d, t, self.qr)
        return (u, d, t, sq)

    def wrap(self, l, g, sigma):
        ev = exp_v_diag(self.field[:, l], self.lamb, sigma)
        g2 = (g / ev[:, None]) * ev[None, :]
        return self.exp_k_inv @ g2 @ self.exp_k

    def sweep(self, uniforms, record=None):
        n, L = self.n, self.L
        ch = chunks(L, self.stab_every)
        stacks = [self.right_stack(+1), self.right_stack(-1)]
        g = []
        for s in range(2):
            gs, ld, sg = green_from_udt(stacks[s][-1], identity_udt(n))
            g.append(gs)
            self.logdet[s], self.sign[s] = ld, sg
        lefts = [identity_udt(n), identity_udt(n)]
        acc_rec = np.zeros((L, n), np.int8)
        rat_rec = np.zeros((L, n))
        self.max_resid = 0.0
        pos = 0
        for c in reversed(range(len(ch))):
            lo, hi = ch[c]
            for l in reversed(range(lo, hi)):
                step = L - 1 - l
                if self.delay > 0:
                    pos = self._update_slice_delayed(g, l, step, uniforms, pos, acc_rec, rat_rec)
                    if l > 0:
                        g = [self.wrap(l, g[0], +1), self.wrap(l, g[1], -1)]
                    continue
                for i in range(n):
                    s_il = self.field[i, l]
                    dl_up = np.exp(2.0 * self.lamb * s_il) - 1.0
                    dl_dn = np.exp(-2.0 * self.lamb * s_il) - 1.0
                    r_up = 1.0 + dl_up * (1.0 - g[0][i, i])
                    r_dn = 1.0 + dl_dn * (1.0 - g[1][i, i])
                    ratio = r_up * r_dn
                    acc = uniforms[pos] <= ratio
                    pos += 1
                    acc_rec[step, i] = acc
                    rat_rec[step, i] = ratio
                    if acc:
                        for s, dl, r in ((0, dl_up, r_up), (1, dl_dn, r_dn)):
                            gg = g[s]
                            x = gg[:, i].copy()
                            y = -gg[i, :].copy()
                            y[i] += 1.0
                            y *= dl / r
                            g[s] = gg - np.outer(x, y)
                        self.field[i, l] = -s_il
                if l > 0:
                    g = [self.wrap(l, g[0], +1), self.wrap(l, g[1], -1)]
            if c > 0:
                for s, sigma in ((0, +1), (1, -1)):
                    lefts[s] = self.left_step(sigma, lefts[s], lo, hi)
                    gs, ld, sg = green_from_udt(stacks[s][c - 1], lefts[s])
                    self.max_resid = max(self.max_resid, float(np.abs(gs - g[s]).max()))
                    g[s] = gs
                    self.logdet[s], self.sign[s] = ld, sg
        self.green = np.stack(g)
        if record is not None:
            record["accept"] = acc_rec
            record["ratio"] = rat_rec
        return self.green


def _slice_rank1(self, g, l, step, uniforms, pos, acc_rec, rat_rec):
    """Site updates of slice l (visit step `step`) with the rank-1 update of ``sweep``."""
    for i in range(self.n):
        s_il = self.field[i, l]
        dl_up = np.exp(2.0 * self.lamb * s_il) - 1.0
        dl_dn = np.exp(-2.0 * self.lamb * s_il) - 1.0
        r_up = 1.0 + dl_up * (1.0 - g[0][i, i])
        r_dn = 1.0 + dl_dn * (1.0 - g[1][i, i])
        ratio = r_up * r_dn
        acc = uniforms[pos] <= ratio
        pos += 1
        acc_rec[step, i] = acc
        rat_rec[step, i] = ratio
        if acc:
            for s, dl, r in ((0, dl_up, r_up), (1, dl_dn, r_dn)):
                gg = g[s]
                x = gg[:, i].copy()
                y = -gg[i, :].copy()
                y[i] += 1.0
                y *= dl / r
                g[s] = gg - np.outer(x, y)
            self.field[i, l] = -s_il
    return pos


def _wrap_up(self, l, g, sigma):
    """G <- B_l G B_l^-1 = exp_v(l) exp_k G exp_k^-1 exp_v(l)^-1 (from slice l-1 to slice l)."""
    ev = exp_v_diag(self.field[:, l], self.lamb, sigma)
    return (ev[:, None] * (self.exp_k @ g @ self.exp_k_inv)) / ev[None, :]


def _right_chunk(self, sigma, prev, lo, hi):
    """UDT of B_{hi-1} ... B_lo R_prev (prev None: identity)."""
    u, d, t, _ = prev if prev is not None else identity_udt(self.n)
    z = u
    for l in range(lo, hi):
        z = self.b_left(l, sigma, z)
    return udt_step(z, d, t, self.qr)


def sweep_alternating(self, uniforms, record=None):
    """One sweep of the alternating order: down (l = L-1 .. 0) and up (l = 0 .. L-1) in
    turn.  A down sweep builds the right stack from scratch only on the first sweep (later
    the previous up sweep's right products serve), stores the left product at every chunk
    boundary, wraps below slice 0 and refreshes G(0) = (1 + B_{L-1} ... B_0)^-1 from the full
    left product; an up sweep wraps into each slice before visiting it
    (G <- B_l G B_l^-1), absorbs each finished chunk into the right product, refreshes at the
    chunk boundaries from (right product, stored left product) and at the top from the full
    right product.  Uniforms and decisions are in visit order."""
    n, L = self.n, self.L
    ch = chunks(L, self.stab_every)
    K = len(ch)
    state = getattr(self, "alt_state", 0)
    acc_rec = np.zeros((L, n), np.int8)
    rat_rec = np.zeros((L, n))
    self.max_resid = 0.0
    pos = 0
    upd = self._update_slice_delayed if self.delay > 0 else self._slice_rank1

    def refresh(s, right, left, g_old):
        gs, ld, sg = green_from_udt(right, left)
        self.max_resid = max(self.max_resid, float(np.abs(gs - g_old).max()))
        self.logdet[s], self.sign[s] = ld, sg
        return gs

    if state != 1:
        if state == 0:
            self.right = [self.right_stack(+1), self.right_stack(-1)]
            g = []
            for s in range(2):
                gs, ld, sg = green_from_udt(self.right[s][-1], identity_udt(n))
                g.append(gs)
                self.logdet[s], self.sign[s] = ld, sg
        else:
            g = [self.green[0].copy(), self.green[1].copy()]
        self.left = [[None] * K, [None] * K]
        for c in reversed(range(K)):
            lo, hi = ch[c]
            for l in reversed(range(lo, hi)):
                pos = upd(g, l, L - 1 - l, uniforms, pos, acc_rec, rat_rec)
                g = [self.wrap(l, g[0], +1), self.wrap(l, g[1], -1)]
            for s, sigma in ((0, +1), (1, -1)):
                prev = self.left[s][c + 1] if c + 1 < K else identity_udt(n)
                self.left[s][c] = self.left_step(sigma, prev, lo, hi)
                right = self.right[s][c - 1] if c > 0 else identity_udt(n)
                g[s] = refresh(s, right, self.left[s][c], g[s])
        self.alt_state = 1
    else:
        g = [self.green[0].copy(), self.green[1].copy()]
        for c in range(K):
            lo, hi = ch[c]
            for l in range(lo, hi):
                g = [self._wrap_up(l, g[0], +1), self._wrap_up(l, g[1], -1)]
                pos = upd(g, l, l, uniforms, pos, acc_rec, rat_rec)
            for s, sigma in ((0, +1), (1, -1)):
                self.right[s][c] = self._right_chunk(sigma, self.right[s][c - 1] if c else None, lo, hi)
                left = self.left[s][c + 1] if c + 1 < K else identity_udt(n)
                g[s] = refresh(s, self.right[s][c], left, g[s])
        self.alt_state = 2
    self.green = np.stack(g)
    if record is not None:
        record["accept"] = acc_rec
        record["ratio"] = rat_rec
    return self.green


Chain._slice_rank1 = _slice_rank1
Chain._wrap_up = _wrap_up
Chain._right_chunk = _right_chunk
Chain.sweep_alternating = sweep_alternating


def _slice_delayed(self, g, l, step, uniforms, pos, acc_rec, rat_rec):
    """Site updates of slice l with delayed rank-k updates: x = G_eff[:, i],
    y = (Delta/R)(e_i - G_eff[i, :]) with G_eff = G - X Y^T; G -= X Y^T every `delay`
    accepted flips and at the end of the slice.  Same ratio, acceptance and uniform per
    site as the rank-1 loop of ``sweep``."""
    n, k = self.n, self.delay
    xs = [np.zeros((n, k)), np.zeros((n, k))]
    ys = [np.zeros((n, k)), np.zeros((n, k))]
    m = 0
    for i in range(n):
        s_il = self.field[i, l]
        dls = (np.exp(2.0 * self.lamb * s_il) - 1.0, np.exp(-2.0 * self.lamb * s_il) - 1.0)
        gii = [g[s][i, i] - xs[s][i, :m] @ ys[s][i, :m] for s in range(2)]
        rs = [1.0 + dls[s] * (1.0 - gii[s]) for s in range(2)]
        ratio = rs[0] * rs[1]
        acc = uniforms[pos] <= ratio
        pos += 1
        acc_rec[step, i] = acc
        rat_rec[step, i] = ratio
        if not acc:
            continue
        for s in range(2):
            x = g[s][:, i] - xs[s][:, :m] @ ys[s][i, :m]
            row = g[s][i, :] - xs[s][i, :m] @ ys[s][:, :m].T
            y = -row
            y[i] += 1.0
            xs[s][:, m] = x
            ys[s][:, m] = y * (dls[s] / rs[s])
        self.field[i, l] = -s_il
        m += 1
        if m == k:
            for s in range(2):
                g[s] = g[s] - xs[s] @ ys[s].T
            m = 0
    if m:
        for s in range(2):
            g[s] = g[s] - xs[s][:, :m] @ ys[s][:, :m].T
    return pos


Chain._update_slice_delayed = _slice_delayed


def green_tau(exp_k, lamb, field, sigma):
    """Unequal-time G_sigma(tau_l, 0) = B_{l-1} ... B_0 (1 + B_{L-1} ... B_0)^-1 for
    l = 0 .. L-1, B_l = exp_v(l) exp_k (the convention of ``Chain``; the reference's get_m,
    lqmc.py:156-185, orders its factors the same way up to the position of exp_v), from the
    field in the reference layout (N, L).  Plain float64 products and one inverse: accurate
    for small beta only.  Returns (L, N, N)."""
    field = np.asarray(field)
    n, L = field.shape
    prods = [np.eye(n)]
    for l in range(L):
        prods.append(exp_v_diag(field[:, l], lamb, sigma)[:, None] * (exp_k @ prods[-1]))
    g0 = np.linalg.inv(np.eye(n) + prods[L])
    return np.stack([prods[l] @ g0 for l in range(L)])


def measure(green, kinetic, u):
    """Equal-time Wick measurements from G_sigma[i, j] = <c_i c+_j> (one sample).

    Returns a dict: density (N,), double_occupancy (N,), kinetic_energy, potential_energy,
    nn (N, N) = <n_i n_j>, szsz (N, N) = <S^z_i S^z_j>."""
    gu, gd = green
    n = gu.shape[0]
    eye = np.eye(n)
    nu = 1.0 - np.diag(gu)
    nd = 1.0 - np.diag(gd)
    out = {}
    out["density"] = nu + nd
    out["double_occupancy"] = nu * nd
    ekin = 0.0
    for g in (gu, gd):
        ekin += np.sum(kinetic * (eye - g.T))
    out["kinetic_energy"] = ekin
    out["potential_energy"] = u * np.sum((nu - 0.5) * (nd - 0.5))
    same = np.zeros((n, n))
    for g, nv in ((gu, nu), (gd, nd)):
        same += np.outer(nv, nv) + (eye - g.T) * g
    cross = np.outer(nu, nd) + np.outer(nd, nu)
    out["nn"] = same + cross
    out["szsz"] = 0.25 * (same - cross)
    return out
