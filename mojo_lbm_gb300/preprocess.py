"""Set-up of flags and boundary values (mirrors src/lbm/preprocess/boundary_condition.mojo:20-309).

Walls are painted into flat arrays in the grid's tiled layout: host numpy arrays here, or device
torch tensors, which the library paints on the GPU (lbm_paint_wall / lbm_paint_wall_values).
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


_SIDE_INDEX = {"-X": 0, "+X": 1, "-Y": 2, "+Y": 3, "-Z": 4, "+Z": 5}


def _on_device(flags, bc) -> bool:
    """True for device torch tensors (painted by the library), False for host numpy arrays."""
    dev = getattr(flags, "is_cuda", False)
    if dev != getattr(bc, "is_cuda", False):
        raise TypeError("flags and bc must both be host arrays or both device tensors")
    return bool(dev)


def set_exterior_walls(grid, config, flags, bc, side: str, boundary_type: int,
                       u=(), rho: float = float("nan"), unitSystem=None, stream=None) -> None:
    """Uniform wall (preprocess/boundary_condition.mojo:78-183).  flags and bc are flat arrays in
    the grid's tiled layout (host numpy, or device tensors painted on the GPU); velocity and density
    are lattice units unless a unitSystem is given."""
    D = grid.D
    u = list(u)
    _error_check(config, D, side, boundary_type, u, rho)
    velocity = [float("nan")] * D if len(u) == 0 else [float(v) for v in u]
    density = float(rho)
    if unitSystem is not None:
        density *= unitSystem.density.C_phys_to_lat()
        velocity = [unitSystem.U.C_phys_to_lat() * v for v in velocity]
    if _on_device(flags, bc):
        import ctypes as C

        from . import _capi
        uv = None if len(u) == 0 else (C.c_float * D)(*velocity)
        _capi.check(_capi.lib().lbm_paint_wall(C.byref(config.to_c()), C.byref(grid.to_c()), _capi.ptr(flags),
                                               _capi.ptr(bc), _SIDE_INDEX[side], int(boundary_type), uv, density,
                                               _capi.stream_ptr(stream)))
        return
    x, y, z = _wall_cells(grid, side)
    lay = grid.layouts
    flags[lay.flag_offset(x, y, z)] = boundary_type
    for i in range(D):
        bc[lay.bc_offset(x, y, z, i)] = velocity[i]
    bc[lay.bc_offset(x, y, z, D)] = density


def set_exterior_walls_with_func(grid, config, flags, bc, side: str, boundary_type: int,
                                 u_func, unitSystem=None, rho: float = float("nan"), stream=None) -> None:
    """Spatially varying wall velocity (preprocess/boundary_condition.mojo:186-309).
    u_func(x, y, z) takes physical coordinates (numpy arrays) and returns D arrays.  With device
    tensors the velocities are evaluated on the host and the wall is painted on the GPU."""
    D = grid.D
    _error_check(config, D, side, boundary_type, [1.0] * D, rho)
    density = float(rho)
    if unitSystem is not None:
        density *= unitSystem.density.C_phys_to_lat()
    conv = unitSystem.U.C_phys_to_lat() if unitSystem is not None else 1.0
    x, y, z = _wall_cells(grid, side)
    px, py, pz = grid.get_grid_coordinates(x, y, z)
    vel = u_func(px, py, pz)
    if _on_device(flags, bc):
        import ctypes as C

        import torch

        from . import _capi
        # face cells with the first free axis fastest (the library's order); _wall_cells makes
        # the last free axis fastest
        axis = _AXES[side[1]]
        free = [a for a in range(3) if a != axis]
        n1, n2 = grid.shape[free[0]], grid.shape[free[1]]
        vals = np.empty((D, n2, n1), np.float32)
        for i in range(D):
            comp = np.broadcast_to(np.asarray(vel[i], dtype=np.float64), x.shape) * conv
            vals[i] = comp.reshape(n1, n2).T
        u_face = torch.from_numpy(vals.reshape(-1)).to(flags.device)
        _capi.check(_capi.lib().lbm_paint_wall_values(C.byref(config.to_c()), C.byref(grid.to_c()),
                                                      _capi.ptr(flags), _capi.ptr(bc), _SIDE_INDEX[side],
                                                      int(boundary_type), _capi.ptr(u_face), density,
                                                      _capi.stream_ptr(stream)))
        if stream is None:
            torch.cuda.current_stream(flags.device).synchronize()  # u_face is released on return
        else:
            stream.synchronize()
        return
    lay = grid.layouts
    flags[lay.flag_offset(x, y, z)] = boundary_type
    for i in range(D):
        bc[lay.bc_offset(x, y, z, i)] = np.broadcast_to(np.asarray(vel[i], dtype=np.float64), x.shape) * conv
    bc[lay.bc_offset(x, y, z, D)] = density
