"""Wall and shape painting on the host, without a GPU: the oracle's restatement of the reference's
painting (oracle/paint.py) against the library's host wall painting and against exact integer
geometry; the sphere's boundary cells; the C ABI's argument checks (they return before any device
work)."""
from __future__ import annotations

import ctypes as C
import itertools
import math

import numpy as np
import pytest

from mojo_lbm_gb300 import Flags, LBM_Config, _capi, preprocess
from mojo_lbm_gb300.geometry import get_sphere_boundary_indices
from oracle import paint
from tests.lbm_cases import make_grid

GRIDS = [("D2Q9", (24, 16, 1), (8, 4, 1)), ("D3Q19", (12, 8, 6), (4, 4, 2)), ("D3Q27", (8, 6, 10), (8, 6, 10))]


@pytest.mark.parametrize("lat,shape,tile", GRIDS)
def test_oracle_walls_equal_host_walls(lat, shape, tile):
    grid = make_grid(lat, shape, tile)
    D = grid.D
    cfg = LBM_Config(BCs={Flags.EQUILIBRIUM})
    rng = np.random.default_rng(4)
    for side, (btype, u, rho) in itertools.product(("-X", "+X", "-Y", "+Y", "-Z", "+Z"),
                                                     [(Flags.SOLID, [0.1, -0.05, 0.02][:D], 1.0),
                                                      (Flags.EQUILIBRIUM, [], 1.02),
                                                      (Flags.EQUILIBRIUM, [0.03] * D, 0.99)]):
        flags0 = rng.integers(0, 3, grid.num_points).astype(np.uint8)
        bc0 = rng.normal(size=grid.num_points * (D + 1)).astype(np.float32)
        f_h, b_h = flags0.copy(), bc0.copy()
        preprocess.set_exterior_walls(grid, cfg, f_h, b_h, side, btype, u, rho)
        f_o, b_o = flags0.copy(), bc0.copy()
        paint.paint_wall(grid.shape, grid.tile_shape, D, f_o, b_o, side, btype,
                         u if u else [math.nan] * D, rho)
        assert np.array_equal(f_h, f_o)
        assert np.array_equal(b_h.view(np.uint32), b_o.view(np.uint32))


def _lattice_ball(shape, D, center, r):
    """Cells of integer distance^2 <= r^2 from an integer centre (exact integer geometry)."""
    X, Y, Z = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    d2 = (X - center[0]) ** 2 + (Y - center[1]) ** 2 + ((Z - center[2]) ** 2 if D == 3 else 0)
    return d2 <= r * r


@pytest.mark.parametrize("lat,shape,tile", GRIDS)
def test_oracle_sphere_and_box_integer_geometry(lat, shape, tile):
    grid = make_grid(lat, shape, tile)
    D = grid.D
    lay = grid.layouts
    X, Y, Z = np.meshgrid(*[np.arange(n) for n in grid.shape], indexing="ij")
    for center, r in [((3, 4, 2), 2), ((0, 0, 0), 3), ((grid.nx - 1, 2, grid.nz - 1), 4), ((5, 3, 1), 0)]:
        c = list(center[:D]) + ([0] if D == 2 else [])
        flags = np.zeros(grid.num_points, np.uint8)
        paint.add_sphere(grid.shape, grid.tile_shape, D, flags, [float(v) for v in c], float(r))
        want = _lattice_ball(grid.shape, D, c, r)
        assert np.array_equal(flags[lay.flag_offset(X, Y, Z)] == 1, want), (center, r)
    flags = np.zeros(grid.num_points, np.uint8)
    half = (2.0, 1.0, 1.0)
    paint.add_box(grid.shape, grid.tile_shape, D, flags, (3.0, 2.0, 1.0 if D == 3 else 0.0), half)
    want = (abs(X - 3) <= 2) & (abs(Y - 2) <= 1) & ((abs(Z - 1) <= 1) if D == 3 else True)
    assert np.array_equal(flags[lay.flag_offset(X, Y, Z)] == 1, want)


@pytest.mark.parametrize("lat,shape", [("D2Q9", (20, 16, 1)), ("D3Q19", (12, 12, 10))])
def test_sphere_boundary_indices(lat, shape):
    grid = make_grid(lat, shape, "untiled")
    D = grid.D
    center = [6.3, 5.8, 4.9 if D == 3 else 0.0]
    flags = np.zeros(grid.num_points, np.uint8)
    ids = get_sphere_boundary_indices(grid, flags, center, 3.1)
    # brute force over the whole grid with the same float32 test
    ref = np.zeros(grid.num_points, np.uint8)
    paint.add_sphere(grid.shape, grid.tile_shape, D, ref, center, 3.1)
    assert np.array_equal(flags, ref)
    lay = grid.layouts
    X, Y, Z = (a.ravel() for a in np.meshgrid(*[np.arange(n) for n in grid.shape], indexing="ij"))
    solid = ref[lay.flag_offset(X, Y, Z)] == 1
    f = np.float32
    hit = np.zeros(X.size, bool)
    for cq in grid.lattice.directions:
        p = [(a + int(cq[k]) if k < D else a).astype(f) for k, a in enumerate((X, Y, Z))]
        s = (p[0] - f(center[0])) * (p[0] - f(center[0])) + (p[1] - f(center[1])) * (p[1] - f(center[1]))
        s = s + (p[2] - f(center[2])) * (p[2] - f(center[2]))
        hit |= s <= f(3.1) * f(3.1)
    want = np.sort(lay.flag_offset(X, Y, Z)[~solid & hit])
    assert np.array_equal(ids, want)
    assert len(ids) > 0


def test_paint_argument_checks_without_a_gpu():
    lib = _capi.lib()
    grid = make_grid("D3Q19", (8, 8, 8), (4, 4, 4)).to_c()
    fake = C.c_void_p(16)  # never dereferenced: every call below fails its checks first
    u = (C.c_float * 3)(0.1, 0.0, 0.0)
    cases = [
        (LBM_Config(), 6, Flags.SOLID, u, 1.0, "Side not valid"),
        (LBM_Config(), 0, Flags.EQUILIBRIUM, u, 1.0, "INCLUDED_BCs"),
        (LBM_Config(), 0, Flags.SOLID, u, math.nan, "both u and rho"),
        (LBM_Config(), 0, Flags.SOLID, None, 1.0, "both u and rho"),
        (LBM_Config(), 0, Flags.FLUID, None, math.nan, "Both cant be left as None"),
        (LBM_Config(include_moving_boundary=False), 0, Flags.SOLID, u, 1.0, "include_moving_boundary"),
        (LBM_Config(BCs={Flags.EQUILIBRIUM}), 0, Flags.EQUILIBRIUM, u, math.nan, "density must also"),
        (LBM_Config(), 0, Flags.FLUID, (C.c_float * 3)(math.nan, 0.0, 0.0), 1.0, "cannot be NaN"),
    ]
    for cfg, side, btype, uu, rho, msg in cases:
        st = lib.lbm_paint_wall(C.byref(cfg.to_c()), C.byref(grid), fake, fake, side, int(btype), uu, rho, None)
        assert st == _capi.LBM_EINVAL and msg in lib.lbm_last_error().decode(), (side, btype, msg)
    c3 = (C.c_float * 3)(1.0, 1.0, 1.0)
    assert lib.lbm_paint_sphere(C.byref(grid), fake, c3, 1.0, c3, 0.0, None) == _capi.LBM_EINVAL
    assert lib.lbm_paint_box(C.byref(grid), fake, c3, None, c3, 1.0, None) == _capi.LBM_EINVAL
    bad = make_grid("D3Q19", (8, 8, 8), (4, 4, 4)).to_c()
    bad.tx = 3
    assert lib.lbm_paint_sphere(C.byref(bad), fake, c3, 1.0, c3, 1.0, None) == _capi.LBM_EINVAL
