"""Post-processing helpers with the reference's names and semantics (lqmc/tools.py)."""
import os

import numpy as np


def get_datapath(filename, model, post='', mkdir=True, **kwargs):
    """Result-file path of a model and run parameters (lqmc/tools.py:12-38).

    The folder is data/u=<u>_t=<t>_mu=<mu>_w=<width>_h=<height> below the working
    directory (created when mkdir), the file "<filename> <k1=v1_k2=v2...><post>.npz"; the
    absolute path is returned.
    """
    width, height = model.lattice.shape
    folder = os.path.join("data", f"u={model.u}_t={model.t}_mu={model.mu}_w={width}_h={height}")
    if mkdir:
        os.makedirs(folder, exist_ok=True)
    params = "_".join(f"{key}={val}" for key, val in kwargs.items())
    return os.path.abspath(os.path.join(folder, f"{filename} {params}{post}.npz"))


def check_params(u, t, dtau):
    """Warn if U t dtau^2 >= 0.1 (lqmc/tools.py:41-60)."""
    check_val = u * t * dtau ** 2
    if check_val < 0.1:
        print(f"Check-value {check_val:.2} is smaller than 0.1!")
    else:
        print(f"Check-value {check_val:.2} should be smaller than 0.1!")


def filling(g_sigma, site=None, axis1=-2, axis2=-1):
    """n = 1 - diag(G) (lqmc/tools.py:63-84)."""
    n = 1 - np.diagonal(g_sigma, axis1=axis1, axis2=axis2)
    if site is not None:
        n = n[..., site]
    return n


def local_moment(gf_up, gf_dn, site=None, axis1=-2, axis2=-1):
    """n_up + n_dn - 2 n_up n_dn from averaged G (lqmc/tools.py:87-109)."""
    n_up = filling(gf_up, site, axis1, axis2)
    n_dn = filling(gf_dn, site, axis1, axis2)
    return n_up + n_dn - 2 * n_up * n_dn


def local_gf(gf):
    return np.diagonal(gf, axis1=-2, axis2=-1)


def matsubara_frequencies(points, beta):
    """Fermionic Matsubara frequencies i w_n = i pi (2 n + 1) / beta for integer points n
    (lqmc/tools.py:125-142; non-integer points raise TypeError)."""
    n = np.asanyarray(points).astype(dtype=int, casting="safe")
    return (2 * n + 1) * (1j * np.pi / beta)


def _softplus(z):
    """log(1 + e^z), elementwise, real or complex, without overflow: the branch on Re z
    keeps the exponential's argument non-positive."""
    z = np.asanyarray(z)
    pos = z.real > 0
    zz = np.where(pos, -z, z)
    return np.where(pos, z, 0) + np.log1p(np.exp(zz))


def fermi_fct(eps, beta):
    """Fermi function 1 / (e^{beta eps} + 1) (lqmc/tools.py:145-162), evaluated as
    exp(-softplus(beta eps)) so that neither sign of beta eps overflows; same type as eps."""
    val = np.exp(-_softplus(beta * np.asanyarray(eps)))
    return val if np.ndim(val) else val[()]


def decompose(a):
    """Eigen-decomposition of the Hermitian matrix a = rv diag(xi) rv_inv
    (lqmc/tools.py:168-170).  rv is unitary, so rv_inv is its conjugate transpose."""
    xi, rv = np.linalg.eigh(a)
    return rv, xi, np.conj(np.swapaxes(rv, -1, -2))


def reconstruct(rv, xi, rv_inv, diag=False):
    """rv diag(xi) rv_inv for every leading index of xi (..., N), or only its diagonal
    (lqmc/tools.py:173-177)."""
    if diag:
        return np.einsum("ik,...k,ki->...i", rv, xi, rv_inv)
    return np.einsum("ik,...k,kj->...ij", rv, xi, rv_inv)


def pole_gf_tau(tau, poles, weights, beta):
    """G(tau) = -sum_p w_p e^{-tau p} / (1 + e^{-beta p}) of a sum of poles, 0 <= tau <= beta
    (lqmc/tools.py:182-190).  Each term is exp(-tau p - softplus(-beta p)), finite for
    either sign of Re p.  tau's shape comes first, then poles' leading axes; the last pole
    axis is summed."""
    assert np.all((tau >= 0.) & (tau <= beta))
    poles, weights = np.atleast_1d(*np.broadcast_arrays(poles, weights))
    tau = np.asanyarray(tau)
    t = tau.reshape(tau.shape + (1,) * poles.ndim)
    terms = np.exp(-t * poles - _softplus(-beta * poles))
    return -np.sum(weights * terms, axis=-1)


def compute_pole_gf_tau(ham, beta):
    """Non-interacting imaginary-time G(tau) of the one-body Hamiltonian ``ham`` on 2049
    points of [0, beta] (lqmc/tools.py:193-200): G(tau) = -V diag(e^{-tau e} / (1 +
    e^{-beta e})) V^T from ham = V diag(e) V^T.  Returns (tau, G) with G of shape
    (N, N, 2049)."""
    energies, vecs = np.linalg.eigh(ham)
    tau = np.linspace(0, beta, num=2049)
    occ = pole_gf_tau(tau, energies[:, None], weights=1, beta=beta)      # (2049, N)
    g = np.einsum("ik,tk,jk->ijt", vecs, occ, np.conj(vecs))
    return tau, g
