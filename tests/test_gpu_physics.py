"""Statistical checks of the GPU dqmc chain against the Trotterised exact diagonalisation.

2x2 periodic Hubbard model (N=4, t=1), U=4, mu=0, beta=2, dtau=0.1 (L=20), stabilisation
every 5 slices, 200 warm-up + 1000 measurement sweeps per chain.  Many independent chains
run batched; the error bar is the spread of the chain means.  At finite dtau the ED of
Tr[O (e^{-dtau V} e^{-dtau K})^L] / Tr[(...)^L] is exact for the estimator the engine uses,
so the QMC must agree within statistics.
"""
import numpy as np
import pytest

from latticeqmc_gb300 import ChainSpec, Engine, HubbardModel
from oracle import ed

pytestmark = pytest.mark.gpu


def test_2x2_observables_match_exact_diagonalisation():
    m = HubbardModel(u=4, t=1, mu=0)
    m.build_square(2)
    K = m.ham_kinetic()
    U, beta, L, n_chains = 4.0, 2.0, 20, 64
    rng = np.random.default_rng(12)
    specs = [ChainSpec(K, U, beta, L, (2 * rng.integers(0, 2, (4, L)) - 1).astype(np.int8))
             for _ in range(n_chains)]
    eng = Engine(specs, mode="dqmc", rng="philox", seed=2020, stab_every=5)
    eng.sweep(200)
    eng.reset_measurements()
    eng.sweep(1000, measure=True)
    obs = [eng.observables(c) for c in range(n_chains)]
    assert not eng.status().any()
    eng.close()
    exact = ed.observables(K, U, beta, L)
    checks = {
        "double_occupancy_mean": exact["double_occupancy"].mean(),
        "kinetic_energy": exact["kinetic_energy"],
        "potential_energy": exact["potential_energy"],
        "density_mean": exact["density"].mean(),
    }
    for key, ref in checks.items():
        vals = np.array([o[key] for o in obs])
        mean, err = vals.mean(), vals.std(ddof=1) / np.sqrt(n_chains)
        assert abs(mean - ref) < 4 * err + 1e-12, f"{key}: {mean:.5f} +- {err:.5f} vs ED {ref:.5f}"
    nn = np.mean([o["nn"] for o in obs], axis=0)
    nn_err = np.std([o["nn"] for o in obs], axis=0, ddof=1) / np.sqrt(n_chains)
    assert np.all(np.abs(nn - exact["nn"]) < 4 * nn_err + 1e-3)
    szsz = np.mean([o["szsz"] for o in obs], axis=0)
    sz_err = np.std([o["szsz"] for o in obs], axis=0, ddof=1) / np.sqrt(n_chains)
    assert np.all(np.abs(szsz - exact["szsz"]) < 4 * sz_err + 1e-3)
