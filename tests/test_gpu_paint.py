"""Wall and shape painting on the device (lbm_paint_*) against the oracle's restatement of the
reference's host painting, bit for bit: every exterior face with fixed, partly free and
function-given values, spheres, circles and boxes (inside, across and outside the grid edges,
with a spacing and origin), on tiled layouts; cells outside the painted set keep their values."""
from __future__ import annotations

import itertools
import math

import numpy as np
import pytest
import torch

from mojo_lbm_gb300 import Flags, LBM_Config, LBM_Grid, preprocess
from mojo_lbm_gb300.geometry import add_box, add_circle, add_sphere
from mojo_lbm_gb300.lattice import get_lattice
from oracle import paint
from tests.lbm_cases import LATTICES, make_grid

pytestmark = pytest.mark.gpu

GRIDS = [("D2Q9", (48, 32, 1), (16, 16, 1)), ("D3Q19", (24, 16, 12), (8, 8, 4)), ("D3Q27", (10, 12, 14), (5, 6, 7))]


def _start(grid, rng):
    flags = rng.integers(0, 4, grid.num_points).astype(np.uint8)
    bc = rng.normal(size=grid.num_points * (grid.D + 1)).astype(np.float32)
    return flags, bc


@pytest.mark.parametrize("lat,shape,tile", GRIDS)
def test_device_walls_equal_oracle(lat, shape, tile):
    grid = make_grid(lat, shape, tile)
    D = grid.D
    cfg = LBM_Config(BCs={Flags.EQUILIBRIUM})
    rng = np.random.default_rng(11)
    for side, (btype, u, rho) in itertools.product(("-X", "+X", "-Y", "+Y", "-Z", "+Z"),
                                                     [(Flags.SOLID, [0.1, -0.05, 0.02][:D], 1.0),
                                                      (Flags.EQUILIBRIUM, [], 1.02),
                                                      (Flags.EQUILIBRIUM, [0.03] * D, 0.99),
                                                      (Flags.FLUID, [0.01] * D, math.nan)]):
        flags, bc = _start(grid, rng)
        fd, bd = torch.from_numpy(flags).cuda(), torch.from_numpy(bc).cuda()
        preprocess.set_exterior_walls(grid, cfg, fd, bd, side, btype, u, rho)
        paint.paint_wall(grid.shape, grid.tile_shape, D, flags, bc, side, btype, u if u else [math.nan] * D, rho)
        assert np.array_equal(fd.cpu().numpy(), flags), (side, btype)
        assert np.array_equal(bd.cpu().numpy().view(np.uint32), bc.view(np.uint32)), (side, btype)


@pytest.mark.parametrize("lat,shape,tile", GRIDS)
def test_device_walls_with_function_equal_host(lat, shape, tile):
    grid = LBM_Grid(get_lattice(LATTICES[lat]), *shape, tile_shape=tile, dx=0.5, origin=(1.0, -2.0, 0.25))
    D = grid.D
    cfg = LBM_Config()

    def u_func(x, y, z):  # a parabolic profile over the other coordinates
        return [0.05 * (1.0 - ((y + z) / 10.0) ** 2), 0.01 * x, 0.02 * z][:D]

    rng = np.random.default_rng(12)
    for side in ("-X", "+X", "-Y", "+Y", "-Z", "+Z"):
        flags, bc = _start(grid, rng)
        fd, bd = torch.from_numpy(flags).cuda(), torch.from_numpy(bc).cuda()
        preprocess.set_exterior_walls_with_func(grid, cfg, fd, bd, side, Flags.SOLID, u_func, rho=1.0)
        preprocess.set_exterior_walls_with_func(grid, cfg, flags, bc, side, Flags.SOLID, u_func, rho=1.0)
        assert np.array_equal(fd.cpu().numpy(), flags), side
        assert np.array_equal(bd.cpu().numpy().view(np.uint32), bc.view(np.uint32)), side


@pytest.mark.parametrize("lat,shape,tile", GRIDS)
@pytest.mark.parametrize("dx,origin", [(1.0, (0.0, 0.0, 0.0)), (0.37, (-1.5, 0.2, 3.0))])
def test_device_shapes_equal_oracle(lat, shape, tile, dx, origin):
    grid = LBM_Grid(get_lattice(LATTICES[lat]), *shape, tile_shape=tile, dx=dx, origin=origin)
    D = grid.D
    rng = np.random.default_rng(13)
    ext = [(n - 1) * dx for n in grid.shape]
    for k in range(12):
        # centres inside, near and beyond the edges; radii from sub-cell to larger than the grid
        center = [origin[i] + rng.uniform(-0.3, 1.3) * ext[i] if i < D else rng.uniform(-1.0, 1.0) for i in range(3)]
        radius = float(rng.choice([0.4, 2.3, 5.0, 40.0])) * dx
        half = [float(rng.uniform(0.2, 6.0)) * dx for _ in range(3)]
        flags = rng.integers(0, 4, grid.num_points).astype(np.uint8)
        fd = torch.from_numpy(flags).cuda()
        if k % 2 == 0:
            (add_circle if D == 2 and k % 4 == 0 else add_sphere)(grid, fd, center, radius)
            paint.add_sphere(grid.shape, grid.tile_shape, D, flags, center, radius, grid.origin, grid.dx)
        else:
            add_box(grid, fd, center, half)
            paint.add_box(grid.shape, grid.tile_shape, D, flags, center, half, grid.origin, grid.dx)
        assert np.array_equal(fd.cpu().numpy(), flags), (k, center, radius, half)


def test_device_painting_builds_a_cavity_the_step_runs():
    """A cavity painted on the device (walls, a moving lid, a sphere) steps bit-exactly like the
    same cavity painted on the host."""
    import oracle
    from mojo_lbm_gb300 import LBM_method
    from mojo_lbm_gb300.solver import Solver
    from tests.test_gpu_step import assert_close, run_both
    grid = make_grid("D3Q19", (16, 16, 8), (8, 8, 4))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER)
    N = grid.num_points
    flags, bc = np.zeros(N, np.uint8), np.zeros(N * 4, np.float32)
    fd, bd = torch.zeros(N, dtype=torch.uint8, device="cuda"), torch.zeros(N * 4, device="cuda")
    for f_, b_ in ((flags, bc), (fd, bd)):
        for s in ("-Y", "+X", "-X", "+Z", "-Z"):
            preprocess.set_exterior_walls(grid, cfg, f_, b_, s, Flags.SOLID, [0.0, 0.0, 0.0], 1.0)
        preprocess.set_exterior_walls(grid, cfg, f_, b_, "+Y", Flags.SOLID, [0.1, 0.0, 0.0], 1.0)
    add_sphere(grid, fd, [8.0, 7.5, 4.0], 2.5)
    paint.add_sphere(grid.shape, grid.tile_shape, 3, flags, [8.0, 7.5, 4.0], 2.5)
    assert np.array_equal(fd.cpu().numpy(), flags)
    assert np.array_equal(bd.cpu().numpy(), bc)
    f0 = np.zeros(N * grid.Q, np.float32)
    oracle.init(cfg, grid, 32, f0)
    got, ref, _, _ = run_both(grid, cfg, fd.cpu().numpy(), bd.cpu().numpy(), f0, 0.8, 6)
    assert_close(got, ref, cfg, "painted cavity")
