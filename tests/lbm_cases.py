"""Seeded test cases shared by the CPU and GPU tests: grids, flags, boundary values and initial
populations in the reference's tiled layout, built on the host."""
from __future__ import annotations

import math

import numpy as np

import oracle
from mojo_lbm_gb300 import Flags, LBM_Config, LBM_Grid, LBM_method, preprocess
from mojo_lbm_gb300.lattice import get_lattice as get_lattice_by_id

LATTICES = {"D2Q9": 0, "D3Q19": 1, "D3Q27": 2}


def make_grid(lattice: str, shape, tile="untiled") -> LBM_Grid:
    return LBM_Grid(get_lattice_by_id(LATTICES[lattice]), *shape, tile_shape=tile)


def ldc_flags(grid: LBM_Grid, cfg: LBM_Config, U: float = 0.1):
    """Closed cavity, lid moving along +x on the +Y wall (examples/LDC.mojo:92-95)."""
    N, D = grid.num_points, grid.D
    flags = np.zeros(N, np.uint8)
    bc = np.zeros(N * (D + 1), np.float32)
    zero = [0.0] * D
    lid = [U] + [0.0] * (D - 1)
    sides = ["-Y", "+X", "-X"] + (["+Z", "-Z"] if D == 3 else [])
    for s in sides:
        preprocess.set_exterior_walls(grid, cfg, flags, bc, s, Flags.SOLID, zero, 1.0)
    preprocess.set_exterior_walls(grid, cfg, flags, bc, "+Y", Flags.SOLID, lid, 1.0)
    return flags, bc


def mixed_flags(grid: LBM_Grid, rng: np.random.Generator):
    """Random flags exercising every branch: SOLID (some with mask bits), EQUILIBRIUM with fixed
    or free (NaN) values, EXCLUDE, capture bits; random wall velocities and densities."""
    N, D = grid.num_points, grid.D
    r = rng.random(N)
    flags = np.zeros(N, np.uint8)
    flags[r < 0.10] = Flags.SOLID
    flags[(r >= 0.10) & (r < 0.12)] = Flags.SOLID | Flags.CAPTURE_DENSITY          # bitmask solid
    flags[(r >= 0.12) & (r < 0.17)] = Flags.EQUILIBRIUM
    flags[(r >= 0.17) & (r < 0.19)] = Flags.FLUID | Flags.EXCLUDE
    flags[(r >= 0.19) & (r < 0.21)] = Flags.FLUID_SOLID_BOUNDARY
    flags[(r >= 0.21) & (r < 0.24)] = Flags.FLUID | Flags.CAPTURE_DENSITY | Flags.CAPTURE_VELOCITY
    bc = np.zeros((N, D + 1), np.float32)
    bc[:, :D] = rng.uniform(-0.05, 0.05, (N, D))
    bc[:, D] = rng.uniform(0.97, 1.03, N)
    # free (NaN) components only on EQUILIBRIUM cells: walls need both u and rho
    # (_error_check, preprocess/boundary_condition.mojo:57-59)
    eq = (flags & 0x0F) == Flags.EQUILIBRIUM
    free_u = eq & (rng.random(N) < 0.3)
    bc[free_u, :D] = np.nan
    free_rho = eq & (rng.random(N) < 0.3)
    bc[free_rho, D] = np.nan
    # bc arrives in cell order (memory order of flags); place in the tiled bc layout
    lay = grid.layouts
    tile = np.arange(N) // lay.T
    loc = np.arange(N) % lay.T
    bcl = np.empty(N * (D + 1), np.float32)
    for k in range(D + 1):
        bcl[loc + lay.T * (k + (D + 1) * tile)] = bc[:, k]
    return flags, bcl


def random_velocity(grid: LBM_Grid, rng: np.random.Generator, amp: float = 0.05):
    """Smooth-ish random velocity field [D, nx, ny, nz] (lattice units)."""
    D = grid.D
    u = np.zeros((D,) + grid.shape)
    X = np.meshgrid(*[np.arange(n) / n for n in grid.shape], indexing="ij")
    for d in range(D):
        for _ in range(3):
            k = rng.integers(1, 3, size=3)
            ph = rng.uniform(0, 2 * math.pi)
            u[d] += amp / 3 * np.sin(2 * math.pi * (k[0] * X[0] + k[1] * X[1] + k[2] * X[2]) + ph)
    return u


def initial_f(grid: LBM_Grid, cfg: LBM_Config, rng: np.random.Generator | None, prec: int = 32, amp: float = 0.05,
              noise: float = 1e-3, tau: float = 0.8):
    """Equilibrium of a random velocity field (+ seeded non-equilibrium noise) in storage form."""
    dt = oracle.f_dtype(cfg, prec)
    f = np.zeros(grid.num_points * grid.Q, dtype=dt)
    if rng is None:
        oracle.init(cfg, grid, prec, f)
        return f
    u = random_velocity(grid, rng, amp)
    if noise == 0.0 or (cfg.use_float16c and prec == 32):
        oracle.init(cfg, grid, prec, f, 1.0, tau, u)
        if noise and cfg.use_float16c and prec == 32:
            # perturb in float, then re-encode
            f32 = oracle.f16c_decode(f) + rng.normal(0, noise * 0.1, f.size).astype(np.float32)
            f = oracle.f16c_encode(f32)
        return f
    oracle.init(cfg, grid, prec, f, 1.0, tau, u)
    f += rng.normal(0, noise, f.size).astype(dt) * (0.1 if prec == 32 else 0.1)
    return f


def fluid_mask_pop(grid: LBM_Grid, flags: np.ndarray) -> np.ndarray:
    """Population-layout mask of cells that are not SOLID (enum) — the cells a step writes
    in the double-buffer method, or that own their slots."""
    lay = grid.layouts
    N = grid.num_points
    tile = np.arange(N) // lay.T
    loc = np.arange(N) % lay.T
    keep = (flags & 0x0F) != Flags.SOLID
    m = np.zeros(N * grid.Q, bool)
    for q in range(grid.Q):
        m[loc + lay.T * (q + grid.Q * tile)] = keep
    return m


def step_case(lat: str, meth: str, store: str, coll: str, les: bool, case: str, shape, tile):
    """A seeded step case, the recipe of the step-parity tests: 'mixed' (random flags over every
    boundary branch, capture bits, EXCLUDE, free NaN bc components) or 'ldc' (closed cavity with a
    moving lid).  Returns (grid, cfg, flags, bc, f0, tau)."""
    import zlib

    grid = make_grid(lat, shape, tile)
    f16 = store == "f16c"
    method = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    seed = zlib.crc32(f"{lat}/{meth}/{store}/{coll}/{les}/{case}".encode())
    rng = np.random.default_rng(seed)
    if case == "mixed":
        cfg = LBM_Config(method, collision_op=coll, LES=les, BCs={Flags.EQUILIBRIUM}, DDF_shift=f16 or bool(seed % 2),
                         use_float16c=f16, capture_density=True, capture_velocity=True)
        flags, bc = mixed_flags(grid, rng)
    else:
        cfg = LBM_Config(method, collision_op=coll, LES=les, DDF_shift=f16, use_float16c=f16)
        flags, bc = ldc_flags(grid, cfg, 0.1)
    tau = 0.55 if coll == "KBC" else 0.8
    f0 = initial_f(grid, cfg, rng, tau=tau)
    return grid, cfg, flags, bc, f0, tau


def digest(*arrays) -> str:
    """SHA-256 of the arrays' bytes, in order (the oracle goldens' digests)."""
    import hashlib

    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()
