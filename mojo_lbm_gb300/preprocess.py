"""Host-side set-up of flags and boundary values
(mirrors src/lbm/preprocess/boundary_condition.mojo:20-309).

Walls are painted into host numpy arrays in the tiled layout; Assembly uploads them.
"""
from __future__ import annotations

import math

import numpy as np

from .constants import Flags, SOLID_NODE

_SIDES = {"-X", "+X", "-Y", "+Y", "-Z", "+Z"}
_AXES = {"X": 0, "Y": 1, "Z": 2}


def _error_check(config, D: int, side: str, boundary_type: int, u, rho: float) -> None:
    """_error_check (preprocess/boundary_condition.mojo:20-69)."""
    if boundary_type not in config.INCLUDED_BCs:
        raise ValueError(f"Input Boundary Type was {boundary_type} but valid boundary types are: "
                         f"{sorted(config.INCLUDED_BCs)}")
    if side not in _SIDES:
        raise ValueError(f"Side not valid. Input was {side} but expects {sorted(_SIDES)}")
    u_is_empty = len(u) == 0
    if u_is_empty and math.isnan(rho):
        raise ValueError("Either velocity or density or both have to be specified. Both cant be left as None")
    if not u_is_empty:
        if len(u) != D:
            raise ValueError(f"Input velocity list was of length {len(u)} but Grid is {D} Dimensional")
        if any(math.isnan(ui) for ui in u):
            raise ValueError("either all components of velocity must be free or specified (cannot be NaN)")
    if boundary_type == SOLID_NODE:
        if u_is_empty or math.isnan(rho):
            raise ValueError("For Solid Type you must specify both u and rho")
        if not config.include_moving_boundary and any(ui != 0.0 for ui in u):
            raise ValueError("include_moving_boundary in config was set to False but a non zero velocity was "
                             "specified, Please set config.include_moving_boundary to True First")
    if boundary_type == Flags.EQUILIBRIUM and not u_is_empty and math.isnan(rho):
        raise ValueError("For Equilibrium BC, if u is specified then the density must also be specified")


def _wall_cells(grid, side: str):
    axis = _AXES[side[1]]
    fixed = 0 if side[0] == "-" else grid.shape[axis] - 1
    rng = [np.arange(n) for n in grid.shape]
    rng[axis] = np.array([fixed])
    x, y, z = np.meshgrid(*rng, indexing="ij")
    return x.ravel(), y.ravel(), z.ravel()


def set_exterior_walls(grid, config, flags: np.ndarray, bc: np.ndarray, side: str, boundary_type: int,
                       u=(), rho: float = float("nan"), unitSystem=None) -> None:
    """Uniform wall (preprocess/boundary_condition.mojo:78-183).  flags and bc are flat host
    arrays in the grid's tiled layout; velocity and density are lattice units unless a
    unitSystem is given."""
    D = grid.D
    u = list(u)
    _error_check(config, D, side, boundary_type, u, rho)
    velocity = [float("nan")] * D if len(u) == 0 else [float(v) for v in u]
    density = float(rho)
    if unitSystem is not None:
        density *= unitSystem.density.C_phys_to_lat()
        velocity = [unitSystem.U.C_phys_to_lat() * v for v in velocity]
    x, y, z = _wall_cells(grid, side)
    lay = grid.layouts
    flags[lay.flag_offset(x, y, z)] = boundary_type
    for i in range(D):
        bc[lay.bc_offset(x, y, z, i)] = velocity[i]
    bc[lay.bc_offset(x, y, z, D)] = density


def set_exterior_walls_with_func(grid, config, flags: np.ndarray, bc: np.ndarray, side: str, boundary_type: int,
                                 u_func, unitSystem=None, rho: float = float("nan")) -> None:
    """Spatially varying wall velocity (preprocess/boundary_condition.mojo:186-309).
    u_func(x, y, z) takes physical coordinates (numpy arrays) and returns D arrays."""
    D = grid.D
    _error_check(config, D, side, boundary_type, [1.0] * D, rho)
    density = float(rho)
    if unitSystem is not None:
        density *= unitSystem.density.C_phys_to_lat()
    conv = unitSystem.U.C_phys_to_lat() if unitSystem is not None else 1.0
    x, y, z = _wall_cells(grid, side)
    px, py, pz = grid.get_grid_coordinates(x, y, z)
    vel = u_func(px, py, pz)
    lay = grid.layouts
    flags[lay.flag_offset(x, y, z)] = boundary_type
    for i in range(D):
        bc[lay.bc_offset(x, y, z, i)] = np.broadcast_to(np.asarray(vel[i], dtype=np.float64), x.shape) * conv
    bc[lay.bc_offset(x, y, z, D)] = density
