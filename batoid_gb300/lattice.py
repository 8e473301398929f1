"""Lattice: an array with primitive lattice vectors (batoid/lattice.py)."""
from functools import cached_property

import numpy as np


def primitiveToLattice(primitiveVectors, Ns):
    """Coordinates n1*a1 + n2*a2 + ... with n_d in [-(N_d//2), N_d - N_d//2)."""
    ns = [np.arange(-(N // 2), -(-N // 2)) for N in Ns]
    ns = np.meshgrid(*ns, indexing='ij')
    return np.matmul(np.moveaxis(ns, 0, -1), primitiveVectors)


class Lattice:
    def __init__(self, array, primitiveVectors):
        primitiveVectors = np.atleast_2d(primitiveVectors)
        if array.ndim != len(primitiveVectors):
            raise ValueError("Not enough primitiveVectors for array")
        if array.ndim != len(primitiveVectors[0]):
            raise ValueError("primitiveVectors are too small for array")
        self.array = array
        self.primitiveVectors = primitiveVectors

    @cached_property
    def coords(self):
        return primitiveToLattice(self.primitiveVectors, self.array.shape)

    def __eq__(self, rhs):
        if not isinstance(rhs, Lattice):
            return False
        return (np.array_equal(self.array, rhs.array)
                and np.array_equal(self.primitiveVectors, rhs.primitiveVectors))

    def __hash__(self):
        return hash(("Lattice", tuple(self.array.ravel()), tuple(self.primitiveVectors.ravel())))

    def __repr__(self):
        return f"Lattice({self.array!r}, {self.primitiveVectors!r})"
