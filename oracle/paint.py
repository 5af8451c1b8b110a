"""Test infrastructure: numpy restatement of the reference's wall and shape painting, the oracle
of the library's device painting (lbm_paint_*).  Not part of the product.

Arrays are flat host arrays in the grid's tiled layout (flags uint8, bc float32 with D+1
components per cell).  Arithmetic is float32, in the reference's operation order.
"""
from __future__ import annotations

import numpy as np

SOLID = 1
_SIDES = ("-X", "+X", "-Y", "+Y", "-Z", "+Z")


def _offsets(tile, shape, x, y, z):
    """Flag offset and tile of cells (x, y, z): lx + tx (ly + ty lz) + T tile (layoutstruct.mojo:37-92)."""
    tx, ty, tz = tile
    ntx, nty = shape[0] // tx, shape[1] // ty
    t = x // tx + ntx * (y // ty + nty * (z // tz))
    loc = x % tx + tx * (y % ty + ty * (z % tz))
    return loc, t, tx * ty * tz


def paint_wall(shape, tile, D, flags, bc, side: str, boundary_type: int, velocity, density):
    """set_exterior_walls (preprocess/boundary_condition.mojo:139-183): every cell of the face gets
    the flag, velocity[0..D-1] and density (NaN = free)."""
    axis = "XYZ".index(side[1])
    fixed = 0 if side[0] == "-" else shape[axis] - 1
    rng = [np.arange(n) for n in shape]
    rng[axis] = np.array([fixed])
    X, Y, Z = (a.ravel() for a in np.meshgrid(*rng, indexing="ij"))
    loc, t, T = _offsets(tile, shape, X, Y, Z)
    flags[loc + T * t] = boundary_type
    for k in range(D):
        bc[loc + T * (k + (D + 1) * t)] = np.float32(velocity[k])
    bc[loc + T * (D + (D + 1) * t)] = np.float32(density)


def paint_wall_values(shape, tile, D, flags, bc, side: str, boundary_type: int, u_face, density):
    """set_exterior_walls_with_func (preprocess/boundary_condition.mojo:253-309) with the velocities
    already evaluated: u_face[k] holds component k per face cell, the first free axis fastest."""
    axis = "XYZ".index(side[1])
    fixed = 0 if side[0] == "-" else shape[axis] - 1
    free = [a for a in range(3) if a != axis]
    n1, n2 = shape[free[0]], shape[free[1]]
    i = np.arange(n1 * n2)
    c = [None, None, None]
    c[axis] = np.full(i.shape, fixed)
    c[free[0]] = i % n1
    c[free[1]] = i // n1
    loc, t, T = _offsets(tile, shape, *c)
    flags[loc + T * t] = boundary_type
    for k in range(D):
        bc[loc + T * (k + (D + 1) * t)] = np.asarray(u_face[k], np.float32)
    bc[loc + T * (D + (D + 1) * t)] = np.float32(density)


def _bbox(shape, D, center, half, origin, dx):
    """The loop bounds of add_sphere / add_box (primatives.mojo:133-138, 220-225)."""
    f = np.float32
    out = []
    for i in range(3):
        if i < D:
            a_min, a_max = f(center[i]) - f(half[i]), f(center[i]) + f(half[i])
            n_min = max(0, int(np.floor((a_min - f(origin[i])) / f(dx))))
            n_max = min(shape[i], int(np.floor((a_max - f(origin[i])) / f(dx)) + f(1)))
            out.append((n_min, n_max))
        else:
            out.append((0, 1))
    return out


def _paint_shape(shape, tile, D, flags, center, half, origin, dx, test):
    f = np.float32
    bb = _bbox(shape, D, center, half, origin, dx)
    if any(hi <= lo for lo, hi in bb):
        return
    X, Y, Z = (a.ravel() for a in np.meshgrid(*[np.arange(lo, hi) for lo, hi in bb], indexing="ij"))
    p = [n.astype(f) * f(dx) + f(origin[k]) for k, n in enumerate((X, Y, Z))]
    ins = test(p)
    loc, t, T = _offsets(tile, shape, X[ins], Y[ins], Z[ins])
    flags[loc + T * t] = SOLID


def add_sphere(shape, tile, D, flags, center, radius, origin=(0.0, 0.0, 0.0), dx=1.0):
    """add_sphere (primatives.mojo:110-186): ((p - c)^2).sum() <= r^2, summed x, y, z in order."""
    f = np.float32
    c = [f(v) for v in center]
    r = f(radius)

    def test(p):
        s = f(0)
        for k in range(3):
            d = p[k] - c[k]
            s = s + d * d
        return s <= r * r

    _paint_shape(shape, tile, D, flags, center, (radius,) * 3, origin, dx, test)


def add_box(shape, tile, D, flags, center, half, origin=(0.0, 0.0, 0.0), dx=1.0):
    """add_box + check_box_axis (primatives.mojo:210-266): center - h <= p <= center + h."""
    f = np.float32
    c = [f(v) for v in center]
    h = [f(v) for v in half]

    def test(p):
        ok = np.ones(p[0].shape, bool)
        for k in range(3):
            ok &= (c[k] - h[k] <= p[k]) & (p[k] <= c[k] + h[k])
        return ok

    _paint_shape(shape, tile, D, flags, center, half, origin, dx, test)
