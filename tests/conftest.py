import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built liblqmc_gpu.so")
    config.addinivalue_line("markers", "slow: long-running statistical test")


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def kinetic_from_golden(side):
    f = golden("kinetic_square.npz")
    n = int(f[f"s{side}_n"])
    k = np.zeros((n, n))
    k[f[f"s{side}_i"], f[f"s{side}_j"]] = f[f"s{side}_v"]
    return k
