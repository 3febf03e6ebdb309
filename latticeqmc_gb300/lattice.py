"""Lattice geometry for the Hubbard model's kinetic matrix.

Drop-in for the part of ``lqmc.Lattice`` (lqmc/lattice.py:283-1033) that the sweep needs:
Bravais lattices with a basis (the reference's prefabs chain, square, hexagonal and cubic,
lqmc/lattice.py:310-421, and ``add_atom`` for others), site numbering, nearest neighbours and
periodic boundaries.  Site numbering follows the reference exactly: the translation vectors
of a lattice of shape ``(s_0, s_1, ...)`` are the points of ``numpy.meshgrid`` over the
ranges, flattened in Fortran order and stably sorted by the first coordinate
(lqmc/lattice.py:226-242, :878-892), with the basis atom fastest; for a 2D ``(width,
height)`` lattice with one atom this is site ``x * height + y``.

Nearest neighbours are the sites at the smallest non-zero distance of the infinite lattice
(distances rounded to 5 decimals, as lqmc/lattice.py:630-632).  Periodic boundaries are
built from the translation vectors: along each periodic axis a site also bonds with the
images of the other sites shifted by the lattice's extent along that axis.  The reference
instead searches for boundary partners by distance and raises ``ValueError`` whenever
``side - 1`` is the hypotenuse of a Pythagorean triple (lqmc/lattice.py:1030-1031: square
sizes 6, 11, 16, ...); this builder has no such restriction and agrees with the reference
on every square size the reference can build.  As in the reference, a periodic axis of
length 2 adds no second bond (the wrap-around partner is already the open-boundary
neighbour).
"""
import itertools

import numpy as np

DIST_DECIMALS = 5


def cell_vectors(shape):
    """Translation vectors of a lattice of the given shape, in the reference's site order."""
    axes = np.meshgrid(*[np.arange(int(s)) for s in shape])
    grid = np.stack([a.flatten("F") for a in axes], axis=1)
    return grid[np.argsort(grid[:, 0], kind="stable")]


def _nearest_only(neighbour_dist):
    if neighbour_dist != 1:
        raise ValueError("only nearest neighbours (neighbour_dist=1) enter the Hubbard kinetic matrix")


class Lattice:
    """Bravais lattice (primitive vectors as columns) with a basis of atoms."""

    def __init__(self, vectors=None, dim=2):
        if vectors is None:
            vectors = np.eye(dim)
        self.vectors = np.asarray(vectors, dtype=np.float64)
        self.dim = self.vectors.shape[0]
        self.atoms = []
        self.atom_positions = []
        self.n_sites = 0
        self.shape = None
        self.indices = None
        self.neighbours = None
        self._periodic = ()

    # -- prefabs (lqmc/lattice.py:310-421) -------------------------------------------------
    @classmethod
    def chain(cls, name="A", a=1.0, neighbour_dist=1, size=None):
        _nearest_only(neighbour_dist)
        latt = cls(np.eye(2) * a)
        latt.add_atom(name)
        if size is not None:
            latt.build((size, 1))
        return latt

    @classmethod
    def square(cls, name="A", a=1.0, neighbour_dist=1, shape=None):
        _nearest_only(neighbour_dist)
        latt = cls(np.eye(2) * a)
        latt.add_atom(name)
        if shape is not None:
            latt.build(shape)
        return latt

    @classmethod
    def hexagonal(cls, atom1="A", atom2="B", a=1.0, neighbour_dist=1, shape=None):
        _nearest_only(neighbour_dist)
        latt = cls(a * np.array([[np.sqrt(3), np.sqrt(3) / 2], [0.0, 3 / 2]]))
        latt.add_atom(atom1)
        latt.add_atom(atom2, pos=[0.0, a])
        if shape is not None:
            latt.build(shape)
        return latt

    @classmethod
    def cubic(cls, name="A", a=1.0, neighbour_dist=1, shape=None):
        _nearest_only(neighbour_dist)
        latt = cls(np.eye(3) * a)
        latt.add_atom(name)
        if shape is not None:
            latt.build(shape)
        return latt

    # -- cell --------------------------------------------------------------------------------
    @property
    def n_base(self):
        return len(self.atoms)

    def add_atom(self, name="A", pos=None):
        """Add a site to the unit cell at `pos` (lqmc/lattice.py:469-496)."""
        pos = np.zeros(self.dim) if pos is None else np.asarray(pos, dtype=np.float64)
        if any(np.all(pos == p) for p in self.atom_positions):
            raise ValueError(f"Position {pos} allready occupied")
        self.atoms.append(name)
        self.atom_positions.append(pos)

    def nearest_distance(self):
        """Smallest non-zero distance between sites of the infinite lattice."""
        if not self.atoms:
            raise ValueError("the lattice has no atoms")
        cells = np.array(list(itertools.product(range(-2, 3), repeat=self.dim)), dtype=np.float64)
        base = np.array(self.atom_positions)
        pts = (cells @ self.vectors.T)[:, None, :] + base[None, :, :]
        d = np.linalg.norm(pts.reshape(-1, 1, self.dim) - base[None, :, :], axis=2)
        d = np.round(d, DIST_DECIMALS)
        return float(np.min(d[d > 0]))

    # -- finite lattice ----------------------------------------------------------------------
    def build(self, shape):
        """Build the open lattice of the given shape (lqmc/lattice.py:894-904)."""
        if not self.atoms:
            self.add_atom()
        shape = tuple(int(s) for s in np.atleast_1d(shape))
        if len(shape) < self.dim:
            shape = shape + (1,) * (self.dim - len(shape))
        if len(shape) != self.dim or min(shape) < 1:
            raise ValueError(f"shape must have {self.dim} positive entries, got {shape}")
        self.shape = np.array(shape)
        cells = cell_vectors(shape)
        nb = self.n_base
        self.indices = np.array([[*c, a] for c in cells for a in range(nb)])
        self.n_sites = len(self.indices)
        self._periodic = ()
        self._rebuild_neighbours()
        return self.indices, self.shape

    def set_periodic_boundary(self, axis=0):
        """Close the lattice along one or several axes (lqmc/lattice.py:994-1033)."""
        if self.shape is None:
            raise ValueError("build the lattice before setting periodic boundaries")
        axes = tuple(int(a) for a in np.atleast_1d(axis))
        for a in axes:
            if a < 0 or a >= self.dim:
                raise ValueError(f"axis {a} out of range for a {self.dim}D lattice")
        self._periodic = tuple(sorted(set(self._periodic) | set(axes)))
        self._rebuild_neighbours()

    def position(self, i):
        """Position of site i."""
        idx = self.indices[i]
        return self.vectors @ idx[:-1] + self.atom_positions[idx[-1]]

    def _rebuild_neighbours(self):
        pos = np.array([self.position(i) for i in range(self.n_sites)])
        d0 = self.nearest_distance()
        # images of the lattice along the periodic axes; bonds found twice (an axis of length
        # 2, whose wrap-around partner is already a neighbour) or to a site's own image (an
        # axis of length 1 in a one-atom cell) merge into the boolean adjacency
        per = list(self._periodic)
        shifts = [np.zeros(self.dim)]
        for combo in itertools.product((-1, 0, 1), repeat=len(per)):
            if any(combo):
                s = np.zeros(self.dim)
                for a, c in zip(per, combo):
                    s += c * self.shape[a] * self.vectors[:, a]
                shifts.append(s)
        adj = np.zeros((self.n_sites, self.n_sites), dtype=bool)
        for s in shifts:
            d = np.linalg.norm(pos[:, None, :] - (pos[None, :, :] + s), axis=2)
            adj |= np.round(np.abs(d - d0), DIST_DECIMALS) == 0.0
        np.fill_diagonal(adj, False)
        adj |= adj.T
        self.neighbours = [[list(np.nonzero(adj[i])[0])] for i in range(self.n_sites)]

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
