"""Lattice velocity sets D2Q9 / D3Q19 / D3Q27 (mirrors src/lbm/lattice.mojo:11-398).

The direction order is the reference's: rest first, then pairs whose second member is the
opposite of the first, which esoteric pull and TRT rely on.
"""
from __future__ import annotations

import numpy as np

D2Q9_ID, D3Q19_ID, D3Q27_ID = 0, 1, 2

_C27 = [
    (0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
    (1, 1, 0), (-1, -1, 0), (1, -1, 0), (-1, 1, 0), (1, 0, 1), (-1, 0, -1), (1, 0, -1), (-1, 0, 1),
    (0, 1, 1), (0, -1, -1), (0, 1, -1), (0, -1, 1),
    (1, 1, 1), (-1, -1, -1), (1, 1, -1), (-1, -1, 1), (1, -1, 1), (-1, 1, -1), (-1, 1, 1), (1, -1, -1),
]
_C9 = [(0, 0), (1, 0), (-1, 0), (0, 1), (0, -1), (1, 1), (-1, -1), (-1, 1), (1, -1)]


def get_stress_indices(D: int) -> list[tuple[int, int]]:
    """Symmetric stress index pairs (lattice.mojo:354-398)."""
    if D == 1:
        return [(0, 0)]
    if D == 2:
        return [(0, 0), (0, 1), (1, 1)]
    if D == 3:
        return [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    raise ValueError("D must be 1, 2 or 3")


class Lattice:
    """Discrete velocities, weights, opposite map and stress pairs of one velocity set."""

    def __init__(self, lattice_id: int, directions, weights):
        self.id = lattice_id
        self.directions = np.asarray(directions, dtype=np.int32)
        self.Q, self.D = self.directions.shape
        self.weights = np.asarray(weights, dtype=np.float64)
        self.float_directions = self.directions.astype(np.float64)
        self.stress_indices = get_stress_indices(self.D)
        self.n_stress_components = len(self.stress_indices)
        self.opposite_indices = np.array(
            [int(np.nonzero((self.directions == -self.directions[i]).all(axis=1))[0][0]) for i in range(self.Q)],
            dtype=np.int32)

    def is_valid_for_esoteric_pull(self) -> bool:
        """Every direction after the rest one is followed by its opposite (lattice.mojo:93-113)."""
        return all((self.directions[q] + self.directions[q + 1] == 0).all() for q in range(1, self.Q - 1, 2))

    def __repr__(self) -> str:
        return f"D{self.D}Q{self.Q}"


def get_D2Q9() -> Lattice:
    w = [4 / 9] + [1 / 9] * 4 + [1 / 36] * 4
    return Lattice(D2Q9_ID, _C9, w)


def get_D3Q19() -> Lattice:
    c = _C27[:19]
    w = [1 / 3] + [1 / 18] * 6 + [1 / 36] * 12
    return Lattice(D3Q19_ID, c, w)


def get_D3Q27() -> Lattice:
    w = [8 / 27] + [2 / 27] * 6 + [1 / 54] * 12 + [1 / 216] * 8
    return Lattice(D3Q27_ID, _C27, w)


def get_lattice(lattice_id: int) -> Lattice:
    return {D2Q9_ID: get_D2Q9, D3Q19_ID: get_D3Q19, D3Q27_ID: get_D3Q27}[lattice_id]()
