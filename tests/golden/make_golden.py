"""Generate the golden fixtures in this folder by running the reference lqmc package.

The reference (KieDani/LatticeQMC, package ``lqmc``) is pure Python.  It is read from
the directory named by the ``LQMC_REFERENCE`` environment variable (required) and imported with stub modules for
matplotlib, which it imports at module top only for plotting
(``lqmc/lattice.py:11-13``, ``lqmc/configuration.py:9``).

Every fixture records the inputs (seed, initial Hubbard-Stratonovich field, the uniform
stream the reference drew) together with the reference's outputs, so that the oracle and
the GPU engine can be replayed against them without the reference present:

* ``kinetic_square.npz``   -- ``HubbardModel.ham_kinetic()`` (``lqmc/hubbard.py:91-110``)
  for every periodic square size the reference can build, stored as sparse triplets.
* ``compat_<s>x<s>.npz``   -- fast sweeps ``LatticeQMC._update_step()`` (``lqmc/lqmc.py:301-347``):
  accept decision and ratio per site, G after every sweep.
* ``det_2x2.npz``          -- determinant-mode sweeps ``_update_step_det`` (``lqmc/lqmc.py:236-259``):
  the exact determinant ratio per site.
* ``run_2x2.npz``          -- a whole ``run_lqmc()`` (``lqmc/lqmc.py:379-393``) with warm-up and
  measurement, its averaged G.
* ``u0_known.npz``         -- the U=0 run against ``tools.compute_pole_gf_tau``
* ``u0_gtau.npz``          -- ``tools.compute_pole_gf_tau`` at the slice times (G(tau, 0))
  (``lqmc/tools.py:193-200``).
* ``exact_chain10_gtau.npz`` -- the reference's own U=0 check (``exact.py:37-54``): a 10-site
  open chain at beta = 4, ``compute_pole_gf_tau`` at the slice times.

Run:  python tests/golden/make_golden.py
"""
import contextlib
import io
import os
import sys
import time
import types

import numpy as np
from scipy.linalg import expm

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("LQMC_REFERENCE")
if not REF:
    raise SystemExit("set LQMC_REFERENCE to the directory that holds the reference's lqmc package")


def _install_matplotlib_stub():
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    coll = types.ModuleType("matplotlib.collections")
    coll.LineCollection = object
    tk = types.ModuleType("mpl_toolkits")
    ag = types.ModuleType("mpl_toolkits.axes_grid1")
    ag.make_axes_locatable = None
    mpl.pyplot = plt
    for name, mod in {"matplotlib": mpl, "matplotlib.pyplot": plt,
                      "matplotlib.collections": coll, "mpl_toolkits": tk,
                      "mpl_toolkits.axes_grid1": ag}.items():
        sys.modules.setdefault(name, mod)


_install_matplotlib_stub()
sys.path.insert(0, REF)
import lqmc  # noqa: E402
from lqmc import HubbardModel, LatticeQMC  # noqa: E402
from lqmc.tools import compute_pole_gf_tau  # noqa: E402


def exp_constants(lamb, n_sites):
    """The four exponentials of the sweep in the reference's own call forms, as computed on
    the machine that made the fixture: exp(arg) for arg = 2*lamb*s, s = +1 / -1
    (lqmc.py:313-323) and the exp_v entries exp(-lamb) / exp(+lamb) (lqmc.py:149-154)."""
    e2p = np.exp(+(2 * lamb * np.int8(1)))
    e2m = np.exp(+(2 * lamb * np.int8(-1)))
    col = np.array(([1, -1] * ((n_sites + 2) // 2))[:max(n_sites, 2)], dtype=np.int8)
    ev = np.exp(-1 * 1 * lamb * col)
    return np.array([e2p, e2m, ev[0], ev[1]], dtype=np.float64)


class _UniformRecorder:
    """Wraps ``np.random.rand`` so every uniform the reference draws is kept."""

    def __init__(self):
        self.values = []
        self._orig = None

    def __enter__(self):
        self._orig = np.random.rand
        orig = self._orig

        def rand(*args):
            v = orig(*args)
            self.values.append(np.asarray(v, dtype=np.float64).ravel().copy())
            return v
        np.random.rand = rand
        return self

    def __exit__(self, *exc):
        np.random.rand = self._orig

    def array(self):
        return np.concatenate(self.values) if self.values else np.zeros(0)


def kinetic_fixtures():
    out = {}
    sizes = [2, 3, 4, 5, 7, 8, 9, 10, 12]
    for s in sizes:
        m = HubbardModel(u=4, t=1, mu=0)
        m.build_square(s)
        k = m.ham_kinetic()
        i, j = np.nonzero(k)
        out[f"s{s}_i"] = i.astype(np.int32)
        out[f"s{s}_j"] = j.astype(np.int32)
        out[f"s{s}_v"] = k[i, j]
        out[f"s{s}_n"] = np.int32(k.shape[0])
    # default chemical potential mu=None -> u/2 on the diagonal (hubbard.py:30, :99-100)
    m = HubbardModel(u=4, t=1)
    m.build_square(3)
    out["s3_mudefault"] = m.ham_kinetic()
    # an open/periodic chain and a rectangle via HubbardModel.build (hubbard.py:60-76)
    m = HubbardModel(u=4, t=1, mu=0)
    m.build(6, 1, 0)
    out["chain6"] = m.ham_kinetic()
    m = HubbardModel(u=4, t=1, mu=0)
    m.build(4, 3, (0, 1))
    out["rect4x3"] = m.ham_kinetic()
    m = HubbardModel(u=4, t=1, mu=0)
    m.build(4, 4, None)
    out["open4x4"] = m.ham_kinetic()
    out["sizes"] = np.array(sizes, dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "kinetic_square.npz"), **out)


def _solver(side, u, beta, L, seed, det_mode=False):
    m = HubbardModel(u=u, t=1, mu=0)
    m.build_square(side)
    np.random.seed(seed)
    q = LatticeQMC(m, beta=beta, time_steps=L, warmup=0, sweeps=0, det_mode=det_mode, log_lvl=None)
    return m, q


def compat_fixture(side, u, beta, L, seed, n_sweeps):
    m, q = _solver(side, u, beta, L, seed)
    field0 = q.config.config.copy()
    rec_acc, rec_ratio = [], []

    def dbg(i, l):
        rec_acc.append(bool(q.acc))
        rec_ratio.append(float(q.ratio))
    q._debug = dbg
    greens = []
    t0 = time.time()
    with _UniformRecorder() as ur:
        for _ in range(n_sweeps):
            gu, gd = q._update_step()
            greens.append(np.stack([gu, gd]))
    dt = time.time() - t0
    N = q.n_sites
    fname = os.path.join(HERE, f"compat_{side}x{side}.npz")
    np.savez_compressed(
        fname, side=side, u=float(u), beta=float(beta), L=L, seed=seed, n_sweeps=n_sweeps,
        kinetic=q.ham_kin, exp_k=q.exp_k, lamb=float(q.lamb), field0=field0,
        consts=exp_constants(q.lamb, N), exp_k_inv=np.linalg.inv(q.exp_k),
        field_end=q.config.config.copy(), uniforms=ur.array(),
        accept=np.array(rec_acc, dtype=np.int8).reshape(n_sweeps, L, N),
        ratio=np.array(rec_ratio).reshape(n_sweeps, L, N),
        green=np.array(greens), seconds=dt)
    print(f"{fname}: {n_sweeps} sweeps in {dt:.1f}s, acceptance {np.mean(rec_acc):.3f}")


def det_fixture(side, u, beta, L, seed, n_sweeps):
    m, q = _solver(side, u, beta, L, seed, det_mode=True)
    field0 = q.config.config.copy()
    rec_acc, rec_ratio = [], []

    def dbg(i, l):
        rec_acc.append(bool(q.acc))
        rec_ratio.append(float(q.ratio))
    q._debug = dbg
    with _UniformRecorder() as ur:
        old = np.linalg.det(q.get_m(0, +1)) * np.linalg.det(q.get_m(0, -1))
        for _ in range(n_sweeps):
            old = q._update_step_det(old)
    N = q.n_sites
    fname = os.path.join(HERE, f"det_{side}x{side}.npz")
    np.savez_compressed(
        fname, side=side, u=float(u), beta=float(beta), L=L, seed=seed, n_sweeps=n_sweeps,
        kinetic=q.ham_kin, exp_k=q.exp_k, lamb=float(q.lamb), field0=field0,
        consts=exp_constants(q.lamb, N), exp_k_inv=expm(q.dtau * q.ham_kin),
        field_end=q.config.config.copy(), uniforms=ur.array(),
        accept=np.array(rec_acc, dtype=np.int8).reshape(n_sweeps, L, N),
        ratio=np.array(rec_ratio).reshape(n_sweeps, L, N))
    print(f"{fname}: acceptance {np.mean(rec_acc):.3f}")


def run_fixture(side, u, beta, L, seed, warmup, sweeps):
    m = HubbardModel(u=u, t=1, mu=0)
    m.build_square(side)
    np.random.seed(seed)
    with _UniformRecorder() as ur:
        # the constructor draws the field with np.random.randint (configuration.py:120-124)
        state = np.random.get_state()
        q = LatticeQMC(m, beta=beta, time_steps=L, warmup=warmup, sweeps=sweeps, log_lvl=None)
        field0 = q.config.config.copy()
        with contextlib.redirect_stdout(io.StringIO()):
            gf = q.run_lqmc()
    fname = os.path.join(HERE, f"run_{side}x{side}.npz")
    np.savez_compressed(fname, side=side, u=float(u), beta=float(beta), L=L, seed=seed,
                        warmup=warmup, sweeps=sweeps, field0=field0, uniforms=ur.array(),
                        green_mean=gf, exp_k=q.exp_k, lamb=float(q.lamb),
                        consts=exp_constants(q.lamb, q.n_sites), kinetic=q.ham_kin,
                        mt_key0=state[1][:4].astype(np.uint32))
    print(f"{fname}: done")


def u0_fixture():
    out = {}
    for side, beta, L in ((2, 2.0, 20), (4, 4.0, 40)):
        m = HubbardModel(u=0, t=1, mu=0)
        m.build_square(side)
        np.random.seed(3)
        q = LatticeQMC(m, beta=beta, time_steps=L, warmup=1, sweeps=2, log_lvl=None)
        with contextlib.redirect_stdout(io.StringIO()):
            gf = q.run_lqmc()
        tau, gtau = compute_pole_gf_tau(m.ham_kinetic(), beta)
        out[f"s{side}_green_ref"] = gf
        out[f"s{side}_pole_tau0"] = -gtau[..., 0]
        out[f"s{side}_beta"] = beta
        out[f"s{side}_L"] = L
        out[f"s{side}_kinetic"] = m.ham_kinetic()
    np.savez_compressed(os.path.join(HERE, "u0_known.npz"), **out)


def u0_gtau_fixture():
    """The reference's non-interacting imaginary-time G (tools.compute_pole_gf_tau,
    tools.py:182-200) at the slice times tau_l = l beta / L (L divides its 2048 intervals),
    negated to G(tau_l, 0) = <c_i(tau_l) c+_j(0)>, shape (L, N, N)."""
    out = {}
    for side, beta, L in ((2, 2.0, 16), (4, 8.0, 64)):
        m = HubbardModel(u=0, t=1, mu=0)
        m.build_square(side)
        tau, gtau = compute_pole_gf_tau(m.ham_kinetic(), beta)
        idx = np.arange(L) * (2048 // L)
        assert np.allclose(tau[idx], np.arange(L) * beta / L)
        out[f"s{side}_gtau"] = -np.moveaxis(gtau[..., idx], -1, 0)
        out[f"s{side}_beta"] = beta
        out[f"s{side}_L"] = L
        out[f"s{side}_kinetic"] = m.ham_kinetic()
    np.savez_compressed(os.path.join(HERE, "u0_gtau.npz"), **out)


def exact_chain_fixture():
    """exact.py:37-54 of the reference: U = 0, t = 1, mu = U/2, a 10-site chain built with
    open boundaries (``build(n_sites, cycling=None)``), beta = 4; its non-interacting G(tau)
    from tools.compute_pole_gf_tau, negated to G(tau_l, 0) at tau_l = l beta / L, L = 32."""
    n_sites, u, t, beta, L = 10, 0, 1, 4.0, 32
    m = HubbardModel(u=u, t=t, mu=u / 2)
    m.build(n_sites, cycling=None)
    ham = m.ham_kinetic()
    tau, gtau = compute_pole_gf_tau(ham, beta)
    idx = np.arange(L) * (2048 // L)
    assert np.allclose(tau[idx], np.arange(L) * beta / L)
    np.savez_compressed(os.path.join(HERE, "exact_chain10_gtau.npz"), kinetic=ham, beta=beta, L=L,
                        gtau=-np.moveaxis(gtau[..., idx], -1, 0))


def lattice_fixtures():
    """Kinetic matrices of the reference's other lattice prefabs (lattice.py:364-421), built
    through HubbardModel with its lattice replaced: hexagonal (two-atom cell) and cubic, open
    boundaries, and the reference's periodic hexagonal lattices where its distance search
    finds the wrap-around bonds."""
    from lqmc.lattice import Lattice as RefLattice
    out = {}
    for shape in [(2, 2), (3, 2), (2, 3), (4, 3)]:
        m = HubbardModel(u=4, t=1, mu=0)
        m.lattice = RefLattice.hexagonal()
        m.lattice.build(shape)
        out["hex_open_%dx%d" % shape] = m.ham_kinetic()
    for shape in [(2, 2, 2), (3, 2, 2), (3, 3, 2)]:
        m = HubbardModel(u=4, t=1, mu=0)
        m.lattice = RefLattice.cubic()
        m.lattice.build(shape)
        out["cubic_open_%dx%dx%d" % shape] = m.ham_kinetic()
    for shape in [(3, 3), (4, 3)]:
        m = HubbardModel(u=4, t=1, mu=0)
        m.lattice = RefLattice.hexagonal()
        m.lattice.build(shape)
        try:
            m.lattice.set_periodic_boundary((0, 1))
            out["hex_pbc_%dx%d" % shape] = m.ham_kinetic()
        except ValueError:
            pass
    np.savez_compressed(os.path.join(HERE, "kinetic_lattices.npz"), **out)


def main():
    which = sys.argv[1:] or ["kinetic", "lattices", "compat", "det", "run", "u0", "u0_gtau",
                             "exact_chain"]
    if "kinetic" in which:
        kinetic_fixtures()
    if "lattices" in which:
        lattice_fixtures()
    if "compat" in which:
        compat_fixture(2, 4.0, 2.0, 20, seed=7, n_sweeps=40)
        compat_fixture(4, 4.0, 4.0, 40, seed=11, n_sweeps=8)
        compat_fixture(8, 4.0, 4.0, 80, seed=5, n_sweeps=2)
    if "det" in which:
        det_fixture(2, 4.0, 2.0, 20, seed=3, n_sweeps=3)
        det_fixture(4, 4.0, 1.0, 10, seed=4, n_sweeps=1)
    if "run" in which:
        run_fixture(2, 4.0, 2.0, 20, seed=1, warmup=20, sweeps=60)
    if "u0" in which:
        u0_fixture()
    if "u0_gtau" in which:
        u0_gtau_fixture()
    if "exact_chain" in which:
        exact_chain_fixture()


if __name__ == "__main__":
    main()
