"""Host-side logic (CPU only): lattice/K builder, configuration, constants, tools, C ABI."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden, kinetic_from_golden
from latticeqmc_gb300 import Configuration, HubbardModel, Lattice
from latticeqmc_gb300 import _native, tools
from latticeqmc_gb300.engine import ChainSpec, exp_constants, hs_coupling
from latticeqmc_gb300 import _split_sweeps


@pytest.mark.parametrize("side", [2, 3, 4, 5, 7, 8, 9, 10, 12])
def test_kinetic_matches_reference(side):
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(side)
    np.testing.assert_array_equal(m.ham_kinetic(), kinetic_from_golden(side))


def test_kinetic_other_shapes_match_reference():
    f = golden("kinetic_square.npz")
    m = HubbardModel(u=4, t=1)
    m.build_square(3)
    np.testing.assert_array_equal(m.ham_kinetic(), f["s3_mudefault"])
    m = HubbardModel(u=4, t=1, mu=0)
    m.build(6, 1, 0)
    np.testing.assert_array_equal(m.ham_kinetic(), f["chain6"])
    m.build(4, 3, (0, 1))
    np.testing.assert_array_equal(m.ham_kinetic(), f["rect4x3"])
    m.build(4, 4, None)
    np.testing.assert_array_equal(m.ham_kinetic(), f["open4x4"])


@pytest.mark.parametrize("side", [6, 11, 16, 32])
def test_periodic_sizes_the_reference_cannot_build(side):
    """lqmc/lattice.py:1030-1031 raises for these sizes; here every site has 4 neighbours."""
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(side)
    k = m.ham_kinetic()
    assert np.array_equal(k, k.T)
    assert set(np.sum(k != 0, axis=1)) == {4}
    # translation invariance: site (x, y) bonds to (x+-1, y), (x, y+-1) modulo side
    for x, y in ((0, 0), (side - 1, side - 1), (side // 2, 1)):
        i = x * side + y
        nbs = {((x + 1) % side) * side + y, ((x - 1) % side) * side + y,
               x * side + (y + 1) % side, x * side + (y - 1) % side}
        assert set(np.nonzero(k[i])[0]) == nbs


def test_lattice_errors():
    with pytest.raises(ValueError):
        Lattice.square().set_periodic_boundary(0)
    with pytest.raises(ValueError):
        Lattice.square(shape=(0, 3))
    with pytest.raises(ValueError):
        Lattice.cubic(shape=(2, 2, 2)).set_periodic_boundary(3)
    with pytest.raises(ValueError):
        Lattice.square(neighbour_dist=2)


def test_configuration_draws_like_reference():
    np.random.seed(4)
    c = Configuration(5, 7)
    np.random.seed(4)
    ref = (2 * np.random.randint(0, 2, size=(5, 7)) - 1).astype(np.int8)
    np.testing.assert_array_equal(c.config, ref)
    assert c.config.dtype == np.int8
    c.update(1, 2)
    assert c[1, 2] == -ref[1, 2]
    assert c.copy() == c
    assert "n_sites=5" in repr(c)


def test_engine_constants_match_reference_forms():
    for name in ("compat_2x2.npz", "compat_4x4.npz", "compat_8x8.npz"):
        f = golden(name)
        dtau = float(f["beta"]) / int(f["L"])
        lamb = hs_coupling(float(f["u"]), dtau)
        assert lamb == float(f["lamb"])
        np.testing.assert_array_equal(exp_constants(lamb, f["field0"].shape[0]), f["consts"])
        spec = ChainSpec(f["kinetic"], float(f["u"]), float(f["beta"]), int(f["L"]), f["field0"])
        np.testing.assert_array_equal(spec.exp_k, f["exp_k"])
    assert hs_coupling(0.0, 0.1) == 0
    np.testing.assert_array_equal(exp_constants(0, 4), np.ones(4))


def test_chainspec_validates_field_shape():
    with pytest.raises(ValueError):
        ChainSpec(np.zeros((4, 4)), 4.0, 1.0, 10, np.ones((4, 9), np.int8))


def test_sweep_split_like_parallel_process_manager():
    per = _split_sweeps(1001, 8)
    assert per.sum() == 1001 and per[0] == 125 + 1 and all(per[1:] == 125)


def test_tools_match_reference_semantics():
    g = np.diag([0.25, 0.5, 0.75])
    np.testing.assert_allclose(tools.filling(g), [0.75, 0.5, 0.25])
    np.testing.assert_allclose(tools.local_moment(g, g), 2 * np.array([0.75, 0.5, 0.25]) * (1 - np.array([0.75, 0.5, 0.25])))
    K = kinetic_from_golden(2)
    tau, gt = tools.compute_pole_gf_tau(K, 2.0)
    f = golden("u0_known.npz")
    np.testing.assert_allclose(-gt[..., 0], f["s2_pole_tau0"], atol=1e-14)
    assert abs(tools.fermi_fct(0.0, 3.0) - 0.5) < 1e-15


def test_get_datapath_like_reference(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(4)
    p = tools.get_datapath("gf", m, post="_tmp", beta=2, L=20)
    folder = tmp_path / "data" / "u=4_t=1_mu=0_w=4_h=4"
    assert p == str(folder / "gf beta=2_L=20_tmp.npz")
    assert folder.is_dir()


def _header_symbols():
    with open(os.path.join(ROOT, "include", "lqmc_gpu.h")) as fh:
        text = fh.read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(lqmc_\w+)\(", text, re.M)))


def test_header_declares_what_binding_binds():
    assert _header_symbols() == sorted(_native.EXPORTED)


def test_library_loads_and_exports_every_declared_symbol():
    if not os.path.exists(_native.LIB_PATH):
        from latticeqmc_gb300 import build
        build.build()
    lib = _native.load()
    for name in _header_symbols():
        assert hasattr(lib, name), name
    assert lib.lqmc_abi_version() == 1
    # no GPU here: creating a handle must fail with an error code, not crash
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        import ctypes
        p = _native.Params()
        h = ctypes.c_void_p()
        rc = lib.lqmc_create(ctypes.byref(p), ctypes.byref(h))
        assert rc in (-1, -2)
        assert lib.lqmc_last_error(None)
    # argument checks that come before any device call
    import ctypes
    p = _native.Params(mode=_native.MODES["compat"], measure_tau=1)
    h = ctypes.c_void_p()
    assert lib.lqmc_create(ctypes.byref(p), ctypes.byref(h)) == -4
    assert b"dqmc" in lib.lqmc_last_error(None)
    p = _native.Params(mode=_native.MODES["dqmc"], measure_tau=2)
    assert lib.lqmc_create(ctypes.byref(p), ctypes.byref(h)) == -1


def test_other_lattices_match_reference_kinetic_matrices():
    """Hexagonal (two-atom cell) and cubic prefabs, open boundaries: K equal to the
    reference's (tests/golden/kinetic_lattices.npz, recorded by make_golden.py)."""
    z = golden("kinetic_lattices.npz")
    for key in z.files:
        kind, bc, dims = key.split("_")
        shape = tuple(int(s) for s in dims.split("x"))
        m = HubbardModel(u=4, t=1, mu=0)
        m.lattice = Lattice.hexagonal() if kind == "hex" else Lattice.cubic()
        m.lattice.build(shape)
        if bc == "pbc":
            m.lattice.set_periodic_boundary(tuple(range(len(shape))))
        np.testing.assert_array_equal(m.ham_kinetic(), z[key], err_msg=key)


def test_periodic_hexagonal_and_cubic_lattices():
    """Periodic boundaries by minimal image: honeycomb sites have 3 bonds, all A-B; simple
    cubic sites have 6 (sizes >= 3; the reference's distance search cannot close these)."""
    for shape in ((3, 3), (4, 3), (5, 4)):
        lat = Lattice.hexagonal(shape=shape)
        lat.set_periodic_boundary((0, 1))
        for i in range(lat.n_sites):
            nbs = lat.nearest_neighbours(i)
            assert len(nbs) == 3
            assert all(lat.indices[j][-1] != lat.indices[i][-1] for j in nbs)
    lat = Lattice.cubic(shape=(3, 4, 3))
    lat.set_periodic_boundary((0, 1, 2))
    a = lat.adjacency()
    assert np.array_equal(a, a.T) and set(a.sum(1)) == {6.0}
    m = HubbardModel(u=4, t=1, mu=0)
    m.lattice = Lattice.cubic()
    m.build(3, 3, None)
    assert m.n_sites == 9


def test_lattice_qmc_forwards_engine_options(monkeypatch):
    import latticeqmc_gb300.lqmc as lqmc_mod
    seen = {}

    class StandIn:
        def __init__(self, chains, **kw):
            seen.update(kw, n_chains=len(chains))

    monkeypatch.setattr(lqmc_mod, "Engine", StandIn)
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(4)
    np.random.seed(0)
    s = lqmc_mod.LatticeQMC(m, 2.0, 20, log_lvl=None, mode="dqmc", precision="fp64e", rng="philox",
                            stab_every=5, seed=7, delay=12, engine="tiled", fp64e_native=("lu",),
                            measure_tau=True)
    s.engine
    assert seen == dict(n_chains=1, mode="dqmc", precision="fp64e", rng="philox", stab_every=5,
                        seed=7, device=0, delay=12, engine="tiled", fp64e_native=("lu",),
                        measure_tau=True)
    plain = lqmc_mod.LatticeQMC(m, 2.0, 20, log_lvl=None)
    assert plain.mode == "compat" and plain.rng == "replay"
    with pytest.raises(ValueError):
        plain.green_tau()


def test_open_chain_kinetic_matches_reference_exact_script():
    """exact.py:43-45 of the reference builds a 10-site chain with open boundaries."""
    m = HubbardModel(u=0, t=1, mu=0)
    m.build(10, cycling=None)
    np.testing.assert_array_equal(m.ham_kinetic(), golden("exact_chain10_gtau.npz")["kinetic"])


@pytest.mark.parametrize("kw", [dict(mode="fast"), dict(precision="fp16"), dict(rng="mt19937"),
                                dict(engine="cluster"), dict(fp64e_native=("wraps",))])
def test_bad_engine_names_raise_value_error_before_any_device_call(kw):
    args = dict(mode="dqmc", precision="fp64", rng="philox", stab_every=5, delay=0, seed=0,
                record=False, device=0)
    args.update(kw)
    with pytest.raises(ValueError):
        _native.Handle(**args)


def test_lattice_qmc_determinant_mode_loops_drive_a_det_engine(monkeypatch):
    import latticeqmc_gb300.lqmc as lqmc_mod
    made = []

    class StandIn:
        def __init__(self, chains, mode, **kw):
            self.mode, self.kw, self.sweeps, self.measured = mode, kw, [], 0
            self.f = chains[0].field.copy()
            made.append(self)

        def set_field(self, c, f):
            self.f = np.array(f, copy=True)

        def field(self, c):
            return self.f.copy()

        def set_uniforms(self, c, u):
            assert u.size % self.f.size == 0

        def sweep(self, k, measure=False):
            self.sweeps.append((k, measure))
            self.f[0, 0] *= -1
            self.measured += k if measure else 0

        def reset_measurements(self):
            self.measured = 0

        def green_sum(self, c):
            n = self.f.shape[0]
            return np.full((2, n, n), 3.0 * self.measured), self.measured

        def diagnostics(self, c):
            return {"logdet": np.array([-1.5, -0.5]), "sign": np.array([1.0, -1.0])}

    monkeypatch.setattr(lqmc_mod, "Engine", StandIn)
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(2)
    np.random.seed(3)
    s = lqmc_mod.LatticeQMC(m, 2.0, 20, warmup=4, sweeps=6, log_lvl=None)
    f0 = s.config.config.copy()
    s.warmup_loop_det()
    eng = made[-1]
    assert eng.mode == "det" and eng.kw["precision"] == "fp64"
    assert sum(k for k, meas in eng.sweeps if not meas) == 4
    assert s.config.config[0, 0] == f0[0, 0] * (-1) ** len(eng.sweeps)
    gf = s.measure_loop_det()
    np.testing.assert_array_equal(gf, np.full((2, 4, 4), 3.0))
    assert abs(s._update_step_det(123.0) - (-np.exp(2.0))) < 1e-12
    assert len(made) == 1                    # one det engine, reused
    s.set_beta(1.0)
    s.warmup_loop_det()
    assert len(made) == 2                    # a new beta rebuilds it


def test_process_managers_drive_the_batched_entry_points(monkeypatch):
    import latticeqmc_gb300 as pkg
    calls = []

    def fake_measure(model, beta, time_steps, warmup, sweeps, cores=None, det_mode=False, **kw):
        calls.append(("measure", beta, time_steps, warmup, sweeps, cores, det_mode, kw))
        n = model.n_sites
        return np.full((n, n), 1.0), np.full((n, n), 2.0)

    def fake_measure_betas(model, betas, time_steps, warmup=500, sweeps=5000, cores=-1,
                           caching=True, det_mode=False, **kw):
        calls.append(("measure_betas", list(betas), time_steps, warmup, sweeps, caching, det_mode))
        n, m = model.n_sites, len(betas)
        return np.zeros((m, n, n)), np.ones((m, n, n))

    monkeypatch.setattr(pkg, "measure", fake_measure)
    monkeypatch.setattr(pkg, "measure_betas", fake_measure_betas)
    model = HubbardModel(u=4, t=1, mu=0)
    model.build_square(2)
    # as lqmc/__init__.py:17-55 uses it
    mgr = pkg.ParallelProcessManager(model, 2.0, 20, 30, False, procs=8, mode="dqmc")
    mgr.set_jobs(1000)
    mgr.run()
    gf = mgr.get_result()
    mgr.terminate()
    assert gf.shape == (2, 4, 4) and gf[0, 0, 0] == 1.0 and gf[1, 0, 0] == 2.0
    assert calls[-1] == ("measure", 2.0, 20, 30, 1000, 8, False, {"mode": "dqmc"})
    # as lqmc/__init__.py:57-96 uses it
    mgr = pkg.SerialProcessManager(model, 20, 50, 400, False, -1, False)
    mgr.set_jobs([1.0, 2.0, 4.0])
    mgr.run(sleep=1.0)
    gf_up, gf_dn = np.swapaxes(mgr.get_result(), 0, 1)
    assert gf_up.shape == (3, 4, 4) and (gf_up == 0).all() and (gf_dn == 1).all()
    assert calls[-1] == ("measure_betas", [1.0, 2.0, 4.0], 20, 50, 400, False, False)


def test_bench_algorithmic_work_matches_the_worked_example():
    """Flops of one sweep of a 16x16 chain (N = 256, L = 80) at acceptance 0.5 with a
    refresh every 10 slices: wraps 8 L N^3, B-chain 4 L N^3, QR 2 (L / n_s) (4/3) N^3,
    updates 4 A N^2 (A accepted flips) = 1.07e10 + 5.4e9 + 3.6e8 + 2.7e9."""
    import sys
    import types
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    n, L = 256, 80
    spec = types.SimpleNamespace(n=n, L=L)
    flops = bench.algorithmic_flops([spec], [0.5 * n * L], 10)
    parts = 8 * L * n ** 3 + 4 * L * n ** 3 + 2 * 8 * (4 / 3) * n ** 3 + 4 * 0.5 * n * L * n ** 2
    assert flops == pytest.approx(parts, rel=1e-12)
    assert flops == pytest.approx(1.07e10 + 5.37e9 + 3.58e8 + 2.68e9, rel=5e-3)


def test_documented_c_caller_compiles_against_the_header(tmp_path):
    """The minimal C caller of the integration guide compiles against include/lqmc_gpu.h."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    with open(os.path.join(ROOT, "INTEGRATION.md")) as fh:
        blocks = re.findall(r"```c\n(.*?)```", fh.read(), re.S)
    assert blocks, "no C example in the integration guide"
    src = tmp_path / "caller.c"
    src.write_text(blocks[0])
    r = subprocess.run([gcc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-I",
                        os.path.join(ROOT, "include"), "-c", str(src), "-o",
                        str(tmp_path / "caller.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _c_layout(tmp_path, struct, fields):
    """sizeof(struct) and offsetof(struct, f) for each field, from the C compiler."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    src = tmp_path / f"{struct}.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "lqmc_gpu.h"\nint main(void) {\n'
                   f'    printf("%zu\\n", sizeof({struct}));\n'
                   + "".join(f'    printf("%zu\\n", offsetof({struct}, {f}));\n' for f in fields)
                   + "    return 0;\n}\n")
    exe = tmp_path / struct
    r = subprocess.run([gcc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    return out[0], out[1:]


def test_ctypes_params_layout_matches_the_c_struct(tmp_path):
    """Every field of the binding's lqmc_params (and of the guide's stub) sits at the C
    compiler's offset, and the sizes agree."""
    import ctypes
    fields = [f for f, _ in _native.Params._fields_]
    size, offsets = _c_layout(tmp_path, "lqmc_params", fields)
    assert size == ctypes.sizeof(_native.Params)
    assert offsets == [getattr(_native.Params, f).offset for f in fields]
    with open(os.path.join(ROOT, "INTEGRATION.md")) as fh:
        stub = re.findall(r"```python\n(.*?)```", fh.read(), re.S)
    names = re.findall(r'\("(\w+)", ctypes\.c_', "".join(b for b in stub if "class Params" in b))
    assert names == fields


def test_static_chain_binding_layout_matches_the_c_struct(tmp_path):
    """The ctypes mirror of lqmc_static_chain that the allocation-free entry point's test
    passes through the C ABI has the C compiler's layout."""
    import ctypes
    from test_zz_no_alloc import StaticChain
    fields = [f for f, _ in StaticChain._fields_]
    size, offsets = _c_layout(tmp_path, "lqmc_static_chain", fields)
    assert size == ctypes.sizeof(StaticChain)
    assert offsets == [getattr(StaticChain, f).offset for f in fields]
