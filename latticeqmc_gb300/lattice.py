"""Lattice geometry for the Hubbard model's kinetic matrix.

Drop-in for the part of ``lqmc.Lattice`` (lqmc/lattice.py:283-1033) that the sweep needs:
site numbering, nearest neighbours and periodic boundaries of chain and rectangular
lattices.  Site numbering follows the reference exactly: the translation vectors of a
``(width, height)`` lattice are enumerated with ``x`` slow and ``y`` fast
(lqmc/lattice.py:226-242, :878-892), so site ``x * height + y``.

Periodic boundaries are built directly from the translation vectors.  The reference
searches for boundary partners by distance and raises ``ValueError`` whenever ``side - 1``
is the hypotenuse of a Pythagorean triple (lqmc/lattice.py:1030-1031: sizes 6, 11, 16,
...); this builder has no such restriction and agrees with the reference on every size the
reference can build.  As in the reference, a periodic axis of length 2 adds no second bond
(the wrap-around partner is already the open-boundary neighbour).
"""
import numpy as np


class Lattice:
    """Square-cell Bravais lattice with one site per cell (chain or rectangle)."""

    def __init__(self, dim=2):
        self.dim = dim
        self.n_sites = 0
        self.shape = None
        self.indices = None
        self.neighbours = None
        self._periodic = ()

    @classmethod
    def square(cls, shape=None):
        latt = cls(2)
        if shape is not None:
            latt.build(shape)
        return latt

    @classmethod
    def chain(cls, size=None):
        latt = cls(2)
        if size is not None:
            latt.build((size, 1))
        return latt

    def build(self, shape):
        """Build the open lattice of the given (width, height) shape (lqmc/lattice.py:894-904)."""
        shape = tuple(int(s) for s in np.atleast_1d(shape))
        if len(shape) == 1:
            shape = (shape[0], 1)
        if len(shape) != 2 or min(shape) < 1:
            raise ValueError(f"shape must be (width, height) with positive entries, got {shape}")
        self.shape = np.array(shape)
        w, h = shape
        self.indices = np.array([[x, y, 0] for x in range(w) for y in range(h)])
        self.n_sites = w * h
        self._periodic = ()
        self._rebuild_neighbours()
        return self.indices, self.shape

    def set_periodic_boundary(self, axis=0):
        """Close the lattice along one or several axes (lqmc/lattice.py:994-1033)."""
        if self.shape is None:
            raise ValueError("build the lattice before setting periodic boundaries")
        axes = tuple(int(a) for a in np.atleast_1d(axis))
        for a in axes:
            if a < 0 or a > 1:
                raise ValueError(f"axis {a} out of range for a 2D lattice")
        self._periodic = tuple(sorted(set(self._periodic) | set(axes)))
        self._rebuild_neighbours()

    def _site(self, x, y):
        return x * int(self.shape[1]) + y

    def _rebuild_neighbours(self):
        w, h = (int(s) for s in self.shape)
        nbs = [set() for _ in range(self.n_sites)]
        for x in range(w):
            for y in range(h):
                i = self._site(x, y)
                for ax, (dx, dy) in enumerate(((1, 0), (0, 1))):
                    size = w if ax == 0 else h
                    for sgn in (1, -1):
                        xx, yy = x + sgn * dx, y + sgn * dy
                        c = xx if ax == 0 else yy
                        if 0 <= c < size:
                            pass
                        elif ax in self._periodic and size > 2:
                            if ax == 0:
                                xx %= w
                            else:
                                yy %= h
                        else:
                            continue
                        j = self._site(xx, yy)
                        if j != i:
                            nbs[i].add(j)
        self.neighbours = [[sorted(s)] for s in nbs]

    def nearest_neighbours(self, i):
        """Indices of the nearest neighbours of site ``i`` (lqmc/lattice.py:768-769)."""
        return self.neighbours[i][0]

    def adjacency(self):
        """(N, N) 0/1 matrix of nearest-neighbour bonds."""
        a = np.zeros((self.n_sites, self.n_sites))
        for i in range(self.n_sites):
            for j in self.nearest_neighbours(i):
                a[i, j] = 1.0
        return a
