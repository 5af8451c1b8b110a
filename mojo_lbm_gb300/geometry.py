"""Immersed sphere/circle geometry and its bounce-back links
(mirrors src/lbm/geometry/rigidSphere.mojo:14-170 and rigidstationary.mojo:21-169), and the solid
shapes of src/lbm/geometry/primatives.mojo:17-266.

Link discovery is host set-up (numpy); the bounce-back itself, the force sum and the shape
painting (add_sphere / add_circle / add_box into a device flag tensor) run on the device through
the library.
"""
from __future__ import annotations

import numpy as np
import torch

from .constants import Flags


def get_q_for_sphere(xf: np.ndarray, xs: np.ndarray, center: np.ndarray, radius: float) -> np.ndarray:
    """Link parameter t in [0, 1] where the segment xf -> xs meets the sphere
    (rigidSphere.mojo:132-170)."""
    f2c = xf - center
    s2f = xs - xf
    a = (s2f * s2f).sum(-1)
    b = (f2c * s2f).sum(-1) * 2
    c = (f2c * f2c).sum(-1) - radius * radius
    sq = np.sqrt(b * b - 4 * a * c)
    t1 = (-b + sq) / (2 * a)
    t2 = (-b - sq) / (2 * a)
    return np.where((t1 >= 0.0) & (t1 <= 1.0), t1, t2)


class RigidStationaryObject:
    """Link lists of one stationary body: fluid node (flag-layout index), direction into the
    wall, wall distance."""

    def __init__(self, grid, unique_fluid_ids, fluid_boundaries, lattice_links, link_distances, device="cuda"):
        self.grid = grid
        self.unique_fluid_ids = np.asarray(unique_fluid_ids, dtype=np.int32)
        self.fluid_boundaries_list = np.asarray(fluid_boundaries, dtype=np.int32)
        self.lattice_links_list = np.asarray(lattice_links, dtype=np.int32)
        self.link_distances_list = np.asarray(link_distances, dtype=np.float32)
        n = len(self.fluid_boundaries_list)
        if len(self.lattice_links_list) != n or len(self.link_distances_list) != n:
            raise ValueError("links_fluid_list, links_direction_list and links_q_dist, should all be the same length")
        dev = torch.device(device)
        self.fluid_boundaries = torch.as_tensor(self.fluid_boundaries_list, device=dev)
        self.lattice_links = torch.as_tensor(self.lattice_links_list, device=dev)
        self.link_distances = torch.as_tensor(self.link_distances_list, device=dev)
        self.link_forces = torch.zeros(max(n, 1) * grid.D, dtype=torch.float32, device=dev)

    def num_links(self) -> int:
        return len(self.fluid_boundaries_list)

    def bounceback(self, solver, f, method: int, compute_force: bool = True, q_min: float = 0.0, stream=None):
        """RigidStationaryObject.bounceback (rigidstationary.mojo:127-153)."""
        solver.linkwise_bounceback(f, self.link_forces, self.fluid_boundaries, self.lattice_links,
                                   self.link_distances, method, compute_force, q_min, stream)

    def sum_force(self, solver, *, in_lattice_units: bool = True, units=None):
        """Float64 device sum of the link forces (rigidstationary.mojo:155-169)."""
        F = solver.sum_link_force(self.link_forces, self.num_links())
        if in_lattice_units:
            return F
        return tuple(units.force.C_lat_to_phys() * v for v in F)


def get_rigid_sphere(grid, flags_host: np.ndarray, center, radius: float, device="cuda") -> RigidStationaryObject:
    """Marks nodes inside the sphere SOLID in flags_host and collects the fluid-to-solid links
    (rigidSphere.mojo:14-129).  Links are ordered by fluid node (x, y, z) then q."""
    if len(center) != 3:
        raise ValueError(f"centre must be a list of 3 floats got a len of {len(center)} instead")
    D, Q = grid.D, grid.Q
    c = np.asarray(center, dtype=np.float64)
    lo, hi = [], []
    for i in range(3):
        if i < D:
            a_min, a_max = c[i] - radius, c[i] + radius
            lo.append(max(0, int((a_min - grid.origin[i]) // grid.dx) - 1))
            hi.append(min(grid.shape[i], int((a_max - grid.origin[i]) // grid.dx + 1) + 1) + 1)
        else:
            lo.append(0)
            hi.append(1)
    rng = [np.arange(lo[i], min(hi[i], grid.shape[i])) for i in range(3)]
    X, Y, Z = np.meshgrid(*rng, indexing="ij")
    X, Y, Z = X.ravel(), Y.ravel(), Z.ravel()
    P = np.stack(grid.get_grid_coordinates(X, Y, Z), -1)
    inside = ((P - c) ** 2).sum(-1) <= radius ** 2
    lay = grid.layouts
    flags_host[lay.flag_offset(X[inside], Y[inside], Z[inside])] = Flags.SOLID
    fx, fy, fz = X[~inside], Y[~inside], Z[~inside]
    xf = P[~inside]
    # every (fluid candidate, direction) pair whose neighbour lies inside the sphere is a link
    cdirs = grid.lattice.directions.astype(np.int64)                      # [Q, D]
    nb = np.stack([fx, fy, fz], -1)[:, None, :].repeat(Q, 1).astype(np.int64)
    nb[..., :D] += cdirs[None, :, :]
    xs = np.stack(grid.get_grid_coordinates(nb[..., 0], nb[..., 1], nb[..., 2]), -1)   # [n, Q, 3]
    hit = ((xs - c) ** 2).sum(-1) <= radius ** 2                          # [n, Q]
    k_idx, q_idx = np.nonzero(hit)                                        # ordered by node, then q
    fid = lay.flag_offset(fx, fy, fz).astype(np.int64)
    ids = fid[k_idx]
    dirs = q_idx
    dists = get_q_for_sphere(xf[k_idx], xs[k_idx, q_idx], c, radius) if len(k_idx) else np.zeros(0)
    uniq = fid[np.unique(k_idx)]
    return RigidStationaryObject(grid, uniq, ids, dirs, dists, device)


def _f32x3(v, what: str):
    import ctypes as C
    v = [float(x) for x in v]
    if len(v) != 3:
        raise ValueError(f"{what} must be a list of 3 floats got a len of {len(v)} instead")
    return (C.c_float * 3)(*v)


def add_sphere(grid, flags, center, radius: float, stream=None) -> None:
    """add_sphere (primatives.mojo:110-186): SOLID in every cell of the device flag tensor whose
    coordinate lies within `radius` of `center` (physical units; float32 test over the reference's
    bounding box)."""
    import ctypes as C

    from . import _capi
    c = _f32x3(center, "centre")
    _capi.check(_capi.lib().lbm_paint_sphere(C.byref(grid.to_c()), _capi.ptr(flags), c, float(radius),
                                             _f32x3(grid.origin, "origin"), float(grid.dx), _capi.stream_ptr(stream)))


def add_circle(grid, flags, center, radius: float, stream=None) -> None:
    """add_circle (primatives.mojo:188-206): add_sphere on a 2D grid."""
    if grid.D != 2:
        raise ValueError("Circle only valid for 2D")
    add_sphere(grid, flags, center, radius, stream)


def add_box(grid, flags, center, box_radius, stream=None) -> None:
    """add_box (primatives.mojo:210-245): SOLID in every cell of the device flag tensor within
    box_radius (half extents) of center along every axis."""
    import ctypes as C

    from . import _capi
    c = _f32x3(center, "centre")
    h = _f32x3(box_radius, "lengths")
    _capi.check(_capi.lib().lbm_paint_box(C.byref(grid.to_c()), _capi.ptr(flags), c, h,
                                          _f32x3(grid.origin, "origin"), float(grid.dx), _capi.stream_ptr(stream)))


def get_sphere_boundary_indices(grid, flags_host: np.ndarray, center, radius: float) -> np.ndarray:
    """get_sphere_boundary_indices (primatives.mojo:17-104): marks the sphere SOLID in the host
    flags and returns the flag-layout indices of the non-solid cells of its bounding box (one cell
    wider) with a lattice neighbour inside it, in ascending order (the reference returns them in
    the order of a hash set)."""
    if len(center) != 3:
        raise ValueError(f"centre must be a list of 3 floats got a len of {len(center)} instead")
    f32 = np.float32
    c = np.asarray(center, f32)
    r = f32(radius)
    dx = f32(grid.dx)
    o = np.asarray(grid.origin, f32)
    lo, hi = [], []
    for i in range(3):
        if i < grid.D:
            n_min = max(0, int(np.floor((c[i] - r - o[i]) / dx)))
            n_max = min(grid.shape[i], int(np.floor((c[i] + r - o[i]) / dx) + f32(1)))
            lo.append(n_min)
            hi.append(min(n_max + 1, grid.shape[i]))  # the reference's n_max + 1 can pass the grid's end
        else:
            lo.append(0)
            hi.append(1)

    def inside(n):
        p = n.astype(f32) * dx + o
        d = p - c
        return ((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]) <= r * r

    rng = [np.arange(lo[i], hi[i]) for i in range(3)]
    X, Y, Z = np.meshgrid(*rng, indexing="ij")
    n = np.stack([X.ravel(), Y.ravel(), Z.ravel()], -1)
    ins = inside(n)
    lay = grid.layouts
    flags_host[lay.flag_offset(*n[ins].T)] = Flags.SOLID
    cand = n[~ins]
    cd = grid.lattice.directions.astype(np.int64)
    hit = np.zeros(len(cand), bool)
    for q in range(grid.Q):
        m = cand.copy()
        m[:, :grid.D] += cd[q]
        hit |= inside(m)
    return np.sort(lay.flag_offset(*cand[hit].T).astype(np.int64))
