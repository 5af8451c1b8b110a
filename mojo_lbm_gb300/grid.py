"""LBM_Grid and its tiled memory layouts (mirrors src/lbm/grid.mojo:55-441 and
src/lbm/layoutstruct.mojo:18-146).

A layout is blocked_product(col_major tile, col_major tiler): per axis the coordinate splits
into (local, tile) with the local index fastest.  A tile equal to the grid is the reference's
untiled column-major layout.
"""
from __future__ import annotations

import numpy as np

from . import _capi
from .lattice import Lattice
from .units import UnitSystem


def set_tile_shape(tile, D: int) -> tuple[int, int, int]:
    """A single tile size t becomes (t, t, 1) in 2D and (t, t, t) in 3D (grid.mojo:372-389)."""
    if isinstance(tile, int):
        return (tile, tile if D >= 2 else 1, tile if D == 3 else 1)
    t = tuple(int(v) for v in tile)
    if len(t) != 3:
        raise ValueError("tile shape must be an int or a 3-tuple")
    return t


class TiledLayouts:
    """Offsets of f (Q per cell), bc (D+1 per cell) and flags in the tiled layout."""

    def __init__(self, D: int, Q: int, shape: tuple[int, int, int], tile: tuple[int, int, int]):
        self.D, self.Q = D, Q
        self.nx, self.ny, self.nz = shape
        self.tx, self.ty, self.tz = tile
        self.ntx, self.nty, self.ntz = self.nx // self.tx, self.ny // self.ty, self.nz // self.tz
        self.T = self.tx * self.ty * self.tz

    def offset(self, x, y, z, k, K: int):
        """Element offset of component k (of K per cell) at (x, y, z); numpy-broadcastable."""
        x, y, z, k = (np.asarray(v, dtype=np.int64) for v in (x, y, z, k))
        tile = x // self.tx + self.ntx * (y // self.ty + self.nty * (z // self.tz))
        loc = x % self.tx + self.tx * (y % self.ty + self.ty * (z % self.tz))
        return loc + self.T * (k + K * tile)

    def f_offset(self, x, y, z, q):
        return self.offset(x, y, z, q, self.Q)

    def bc_offset(self, x, y, z, k):
        return self.offset(x, y, z, k, self.D + 1)

    def flag_offset(self, x, y, z):
        return self.offset(x, y, z, 0, 1)

    def _perm(self, K: int) -> np.ndarray:
        x, y, z, k = np.meshgrid(np.arange(self.nx), np.arange(self.ny), np.arange(self.nz), np.arange(K),
                                 indexing="ij")
        return self.offset(x, y, z, k, K)

    def to_layout(self, natural: np.ndarray) -> np.ndarray:
        """[nx, ny, nz] or [nx, ny, nz, K] array -> flat array in the tiled layout."""
        a = np.asarray(natural)
        if a.ndim == 3:
            a = a[..., None]
        K = a.shape[3]
        out = np.empty(a.size, dtype=a.dtype)
        out[self._perm(K).ravel()] = a.ravel()
        return out

    def from_layout(self, flat: np.ndarray, K: int) -> np.ndarray:
        """Flat tiled-layout array -> [nx, ny, nz, K] array."""
        a = np.asarray(flat).reshape(-1)
        return a[self._perm(K)]


class LBM_Grid:
    """Shape, tile and lattice of one domain, plus unit-system factories (grid.mojo:55-277)."""

    def __init__(self, lattice: Lattice, nx: int, ny: int, nz: int, tile_shape="untiled", dx: float = 1.0,
                 origin=(0.0, 0.0, 0.0)):
        self.lattice = lattice
        self.D, self.Q = lattice.D, lattice.Q
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.shape = (self.nx, self.ny, self.nz)
        grid_D = (self.nx > 1) + (self.ny > 1) + (self.nz > 1)
        if grid_D != self.D:
            raise ValueError("The given dimension of the Lattice does not match that of the dimension of the grid")
        # "untiled" is the column-major layout of layoutstruct.mojo:67-69 (one tile = the grid);
        # a (1, 1, 1) tile is the per-cell (AoS) blocked_product layout.
        t = self.shape if tile_shape == "untiled" else set_tile_shape(tile_shape, self.D)
        if any(n % ti for n, ti in zip(self.shape, t)):
            raise ValueError("Tile size must divide nx,ny and nz")
        self.tile_shape = t
        self.layouts = TiledLayouts(self.D, self.Q, self.shape, t)
        self.num_points = self.nx * self.ny * self.nz
        self.dx = float(dx)
        self.origin = tuple(float(o) for o in origin)
        self.domain_size = tuple((n - 1) * self.dx for n in self.shape)

    def get_grid_coordinates(self, i, j, k):
        return tuple(np.asarray(idx) * self.dx + o for idx, o in zip((i, j, k), self.origin))

    def get_UnitSystem_with_Re(self, U_phys: float, U_lattice: float, L_phys: float, Re: float,
                               density: float = 1.0) -> UnitSystem:
        L_lattice = L_phys / self.dx
        nu = U_phys * L_phys / Re
        return UnitSystem(U_phys, U_lattice, L_phys, L_lattice, density, nu, self.D)

    def get_UnitSystem(self, U_phys: float, U_lattice: float, L_phys: float, kinematic_viscosity: float,
                       density: float = 1.0) -> UnitSystem:
        return UnitSystem(U_phys, U_lattice, L_phys, L_phys / self.dx, density, kinematic_viscosity, self.D)

    def get_UnitSystem_with_tau(self, U_phys: float, tau: float, L_phys: float, kinematic_viscosity: float,
                                density: float = 1.0, *, min_u: float = 0.001, max_u: float = 0.1) -> UnitSystem:
        L_lattice = L_phys / self.dx
        v_lat = (tau - 0.5) * (1 / 3.0)
        Re = U_phys * L_phys / kinematic_viscosity
        U_lattice = v_lat * Re / L_lattice
        if U_lattice < min_u or U_lattice > max_u:
            raise ValueError(f"Target Tau of {tau} does not satisfy bounds. Calculated u lattice = {U_lattice} "
                             f"which is outside the given bounds of [{min_u} {max_u}]")
        return UnitSystem(U_phys, U_lattice, L_phys, L_lattice, density, kinematic_viscosity, self.D)

    def to_c(self) -> _capi.lbm_grid_t:
        g = _capi.lbm_grid_t()
        g.lattice = self.lattice.id
        g.nx, g.ny, g.nz = self.shape
        g.tx, g.ty, g.tz = self.tile_shape
        return g

    def __repr__(self) -> str:
        return f"LBM_Grid({self.lattice!r}, {self.shape}, tile={self.tile_shape})"
