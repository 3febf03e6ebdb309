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
    n_points = np.asanyarray(points).astype(dtype=int, casting="safe")
    return 1j * np.pi / beta * (2 * n_points + 1)


def fermi_fct(eps, beta):
    """1 / (exp(beta eps) + 1) (lqmc/tools.py:145-162)."""
    return 0.5 * (1. + np.tanh(-0.5 * beta * eps))


def decompose(a):
    xi, rv = np.linalg.eigh(a)
    return rv, xi, np.linalg.inv(rv)


def reconstruct(rv, xi, rv_inv, diag=False):
    if diag:
        return ((np.transpose(rv_inv) * rv) @ xi[..., np.newaxis])[..., 0]
    return (rv * xi[..., np.newaxis, :]) @ rv_inv


def pole_gf_tau(tau, poles, weights, beta):
    """Imaginary-time G of a sum of poles (lqmc/tools.py:182-190)."""
    assert np.all((tau >= 0.) & (tau <= beta))
    poles, weights = np.atleast_1d(*np.broadcast_arrays(poles, weights))
    tau = np.asanyarray(tau)
    tau = tau.reshape(tau.shape + (1,) * poles.ndim)
    exponent = np.where(poles.real >= 0, -tau, beta - tau) * poles
    single_pole_tau = np.exp(exponent) * fermi_fct(-np.sign(poles.real) * poles, beta)
    return -np.sum(weights * single_pole_tau, axis=-1)


def compute_pole_gf_tau(ham, beta):
    """Non-interacting G(tau) of the one-body Hamiltonian ``ham`` (lqmc/tools.py:193-200)."""
    rv, xi, rv_inv = decompose(ham)
    tau = np.linspace(0, beta, num=2049)
    diag_gf_tau = pole_gf_tau(tau, xi[..., np.newaxis], weights=1, beta=beta)
    gf_tau = reconstruct(rv, diag_gf_tau, rv_inv)
    gf_tau = np.moveaxis(gf_tau, 0, -1)
    return tau, gf_tau
