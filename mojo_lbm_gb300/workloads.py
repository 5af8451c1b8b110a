"""Set-up of the benchmark configurations: lid-driven cavities and batches of 2D cylinder
channels (host arrays in the reference's tiled layout; device work happens in the library)."""
from __future__ import annotations

import numpy as np

from .config import LBM_Config
from .constants import Bounceback_method, Flags, LBM_method
from .geometry import get_rigid_sphere
from .grid import LBM_Grid
from .lattice import get_D2Q9
from . import preprocess


def cavity(grid: LBM_Grid, cfg: LBM_Config, U: float):
    """Closed cavity, lid moving along +x on the +Y wall (examples/LDC.mojo:92-95)."""
    N, D = grid.num_points, grid.D
    flags = np.zeros(N, np.uint8)
    bc = np.zeros(N * (D + 1), np.float32)
    sides = ["-Y", "+X", "-X"] + (["+Z", "-Z"] if D == 3 else [])
    for s in sides:
        preprocess.set_exterior_walls(grid, cfg, flags, bc, s, Flags.SOLID, [0.0] * D, 1.0)
    preprocess.set_exterior_walls(grid, cfg, flags, bc, "+Y", Flags.SOLID, [U] + [0.0] * (D - 1), 1.0)
    return flags, bc


class Channel:
    """One 2D channel with a circular cylinder: parabolic moving-wall inlet on -X, equilibrium
    outlet (rho = 1, u free) on +X, no-slip walls on +-Y, Bouzidi links on the cylinder
    (the set-up of benchmarks/Cylinder2D/CylinderFlow_Re20.mojo:143-151, in lattice units)."""

    def __init__(self, nx: int, ny: int, Re: float, u_max: float, y_offset: float, tile=(16, 16, 1)):
        self.grid = LBM_Grid(get_D2Q9(), nx, ny, 1, tile)
        self.cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, BCs={Flags.EQUILIBRIUM})
        N = self.grid.num_points
        self.flags = np.zeros(N, np.uint8)
        self.bc = np.zeros(N * 3, np.float32)
        H = ny - 1.0
        g, c = self.grid, self.cfg
        preprocess.set_exterior_walls(g, c, self.flags, self.bc, "+X", Flags.EQUILIBRIUM, [], 1.0)
        preprocess.set_exterior_walls_with_func(g, c, self.flags, self.bc, "-X", Flags.SOLID,
                                                lambda x, y, z: (4.0 * u_max * y * (H - y) / (H * H), 0.0 * y),
                                                None, 1.0)
        preprocess.set_exterior_walls(g, c, self.flags, self.bc, "-Y", Flags.SOLID, [0.0, 0.0], 1.0)
        preprocess.set_exterior_walls(g, c, self.flags, self.bc, "+Y", Flags.SOLID, [0.0, 0.0], 1.0)
        self.diameter = 0.1 * ny
        self.center = (0.2 * nx, 0.5 * ny + y_offset * ny, 0.0)
        self.body = get_rigid_sphere(g, self.flags, self.center, 0.5 * self.diameter, device="cpu")
        # nu from the mean inlet velocity 2/3 u_max and the diameter (DFG convention)
        self.Re = Re
        self.tau = 3.0 * (2.0 / 3.0 * u_max) * self.diameter / Re + 0.5


def channel_specs(n: int = 512, seed: int = 0, nx_range=(200, 800), granule=(16, 16)):
    """(nx, ny, Re, y_offset) of the batched cylinder-channel workload: nx ~ U[200, 800],
    ny = 0.41 nx, Re ~ U[20, 200], cylinder offset ~ U[-0.05, 0.05] ny; nx and ny rounded to
    multiples of the granule (so that every tile dividing the granule divides every domain)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx = int(rng.integers(nx_range[0], nx_range[1] + 1))
        nx = max(granule[0], int(round(nx / granule[0])) * granule[0])
        ny = max(granule[1], int(round(0.41 * nx / granule[1])) * granule[1])
        out.append((nx, ny, float(rng.uniform(20.0, 200.0)), float(rng.uniform(-0.05, 0.05))))
    return out


def cylinder_channels(n: int = 512, seed: int = 0, nx_range=(200, 800), u_max: float = 0.05, tile=(16, 16, 1),
                      granule=None, specs=None):
    """The channels of channel_specs (granule defaults to the tile) in the given tile layout."""
    specs = specs or channel_specs(n, seed, nx_range, granule or tile[:2])
    return [Channel(nx, ny, Re, u_max, off, tile) for nx, ny, Re, off in specs]


def links_of(channels, device="cuda"):
    """Concatenated link arrays (domain, fluid id, direction, distance) of a list of channels."""
    import torch
    dom = np.concatenate([np.full(ch.body.num_links(), i, np.int32) for i, ch in enumerate(channels)])
    ids = np.concatenate([ch.body.fluid_boundaries_list for ch in channels]).astype(np.int32)
    dirs = np.concatenate([ch.body.lattice_links_list for ch in channels]).astype(np.int32)
    dists = np.concatenate([ch.body.link_distances_list for ch in channels]).astype(np.float32)
    t = lambda a: torch.from_numpy(a).to(device)  # noqa: E731
    return t(dom), t(ids), t(dirs), t(dists), Bounceback_method.BOUZIDI
