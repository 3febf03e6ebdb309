"""Hubbard-Stratonovich field: int8 (n_sites, time_steps) array of +-1.

Same interface as ``lqmc.Configuration`` (lqmc/configuration.py:86-160) without its
plotting helpers.  ``initialize`` draws ``2 * np.random.randint(0, 2, (N, L)) - 1`` from
numpy's global generator, exactly as the reference (configuration.py:120-124), so a solver
constructed after ``np.random.seed(s)`` starts from the reference's field.  The GPU holds
the field as [slice][site]; the transpose happens at the C-ABI boundary.
"""
import numpy as np


class Configuration:

    dtype = np.int8

    def __init__(self, n_sites, time_steps, array=None):
        self.n_sites = n_sites
        self.time_steps = time_steps
        if array is not None:
            self.config = np.asarray(array, dtype=self.dtype)
        else:
            self.initialize()

    def copy(self):
        return Configuration(self.n_sites, self.time_steps, array=self.config.copy())

    def initialize(self):
        config = 2 * np.random.randint(0, 2, size=(self.n_sites, self.time_steps)) - 1
        self.config = config.astype(self.dtype)

    def update(self, i, t):
        self.config[i, t] *= -1

    def get(self, i, t):
        return self.config[i, t]

    def mean(self):
        return np.mean(self.config)

    def var(self):
        return np.var(self.config)

    def __eq__(self, other):
        return np.all(self.config == other.config)

    def __getitem__(self, item):
        return self.config[item]

    def __repr__(self):
        return (f"Configuration(n_sites={self.n_sites}, time_steps={self.time_steps}, "
                f"mean={float(np.mean(self.config)):+.3f})")
