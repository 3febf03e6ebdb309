"""Oracle: Trotterised Fock-space exact diagonalisation (TEST INFRASTRUCTURE ONLY).

The reference has no interacting exact diagonalisation (its exact.py treats U=0 only,
lqmc/tools.py:182-200), so this is project-written.  For a cluster of N sites (2N
fermionic modes, 4**N states) it builds

    K^ = sum_sigma sum_ij K_ij c+_{i sigma} c_{j sigma}        (K from ham_kinetic)
    V^ = U sum_i (n_{i up} - 1/2)(n_{i dn} - 1/2)              (the form the discrete
                                                               HS split of lqmc.py:105 decouples)
    A  = exp(-dtau V^) exp(-dtau K^)

and returns <O> = Tr[O A^L] / Tr[A^L] for equal-time observables.  With A in this order
the operator O sits just left of exp(V_0) in the product exp(V_0) exp(-dtau K) exp(V_{L-1})
... exp(-dtau K) -- the insertion point of the engine's measured Green's function
G = (1 + B_0 B_{L-1} ... B_1)^-1 with B_l = exp(V_l) exp(-dtau K).  So at finite dtau the
comparison carries no Trotter bias: DQMC and this ED agree to statistical error.
"""
import numpy as np
from scipy.linalg import expm


def _operators(n_sites):
    n_modes = 2 * n_sites
    dim = 1 << n_modes
    states = np.arange(dim)
    ops = []
    for m in range(n_modes):
        c = np.zeros((dim, dim))
        occ = (states >> m) & 1
        below = np.array([bin(s & ((1 << m) - 1)).count("1") for s in states])
        sign = np.where(below % 2, -1.0, 1.0)
        src = states[occ == 1]
        c[src ^ (1 << m), src] = sign[occ == 1]
        ops.append(c)
    return ops  # mode index = sigma * n_sites + i, sigma 0 = up, 1 = down


def observables(kinetic, u, beta, time_steps):
    """Exact Trotterised expectation values for the cluster with hopping matrix ``kinetic``."""
    kinetic = np.asarray(kinetic, dtype=np.float64)
    n = kinetic.shape[0]
    dtau = beta / time_steps
    c = _operators(n)
    cd = [x.T for x in c]
    num = [cd[m] @ c[m] for m in range(2 * n)]
    dim = c[0].shape[0]
    hk = np.zeros((dim, dim))
    for s in range(2):
        for i in range(n):
            for j in range(n):
                if kinetic[i, j] != 0.0:
                    hk += kinetic[i, j] * (cd[s * n + i] @ c[s * n + j])
    eye = np.eye(dim)
    hv = np.zeros((dim, dim))
    for i in range(n):
        hv += u * (num[i] - 0.5 * eye) @ (num[n + i] - 0.5 * eye)
    a = expm(-dtau * hv) @ expm(-dtau * hk)
    p = np.linalg.matrix_power(a, time_steps)
    z = np.trace(p)

    def ev(op):
        return float(np.trace(op @ p) / z)

    out = {}
    out["density"] = np.array([ev(num[i] + num[n + i]) for i in range(n)])
    out["double_occupancy"] = np.array([ev(num[i] @ num[n + i]) for i in range(n)])
    out["kinetic_energy"] = ev(hk)
    out["potential_energy"] = ev(hv)
    nn = np.zeros((n, n))
    szsz = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            ni = num[i] + num[n + i]
            nj = num[j] + num[n + j]
            si = num[i] - num[n + i]
            sj = num[j] - num[n + j]
            nn[i, j] = ev(ni @ nj)
            szsz[i, j] = 0.25 * ev(si @ sj)
    out["nn"] = nn
    out["szsz"] = szsz
    g = np.zeros((2, n, n))
    for s in range(2):
        for i in range(n):
            for j in range(n):
                g[s, i, j] = ev(c[s * n + i] @ cd[s * n + j])
    out["green"] = g
    return out
