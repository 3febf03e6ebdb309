"""Hubbard model: interaction, hopping, chemical potential and the kinetic matrix.

Same interface and conventions as ``lqmc.HubbardModel`` (lqmc/hubbard.py:12-110):
``mu=None`` means ``u / 2`` (hubbard.py:30), ``ham_kinetic()`` puts ``-mu`` on the diagonal
and assigns ``-t`` to every nearest-neighbour pair (assigned, not added: hubbard.py:106-110).
"""
import numpy as np

from .lattice import Lattice


class HubbardModel:

    def __init__(self, u=4, t=1, mu=None):
        self.lattice = Lattice.square()
        self.u = u
        self.t = t
        self.mu = mu if mu is not None else u / 2

    def set_params(self, u, t=1.0, mu=None):
        self.u = u
        self.t = t
        self.mu = mu if mu is not None else u / 2

    def param_str(self):
        return f"u={self.u}_t={self.t}_mu={self.mu}"

    def __str__(self):
        return f"HubbardModel(u={self.u}, t={self.t}, mu={self.mu})"

    @property
    def n_sites(self):
        """int: total number of lattice sites."""
        return self.lattice.n_sites

    def build(self, width, height=1, cycling=0):
        """Build a (width, height) lattice, periodic along ``cycling`` (hubbard.py:60-76)."""
        self.lattice.build((width, height))
        if cycling is not None:
            self.lattice.set_periodic_boundary(cycling)

    def build_square(self, size, cycling=(0, 1)):
        """Build a size x size lattice, periodic along both axes by default (hubbard.py:78-89)."""
        self.build(size, size, cycling)

    def ham_kinetic(self):
        """(N, N) float64 kinetic matrix K (hubbard.py:91-110)."""
        n = self.lattice.n_sites
        ham = -self.mu * np.eye(n, dtype=np.float64)
        for i in range(n):
            for j in self.lattice.nearest_neighbours(i):
                if i > j:
                    ham[i, j] = -self.t
                    ham[j, i] = -np.conj(self.t)
        return ham
