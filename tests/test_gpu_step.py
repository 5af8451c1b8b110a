"""Parity of the CUDA step (through the C ABI) with the float32 CPU oracle.

Every lattice x streaming method x storage x collision operator x LES, on two seeded cases:
'mixed' (random flags covering every boundary branch, capture bits and EXCLUDE, random bc with
free NaN components) and 'ldc' (closed cavity with a moving lid).  Grids use non-power-of-two
tiles so the layout decode is exercised.

Tolerance: none.  The library is compiled with --fmad=false and performs every float32 operation
in the oracle's order, so populations (float32 words or Float16C codes), captured bc values and
all auxiliary outputs are compared bit for bit.
"""
from __future__ import annotations

import itertools
import zlib

import numpy as np
import pytest
import torch

import oracle
from mojo_lbm_gb300 import Flags, LBM_Config, LBM_method
from mojo_lbm_gb300.solver import Solver
from tests.lbm_cases import initial_f, ldc_flags, make_grid, mixed_flags

pytestmark = pytest.mark.gpu

STEPS = 6
# generic kernel: non-power-of-two tiles; block-per-tile kernel: 256-cell power-of-two tiles
SHAPES = {"D2Q9": ((30, 20, 1), (10, 5, 1)), "D3Q19": ((18, 12, 10), (6, 4, 5)), "D3Q27": ((12, 12, 10), (4, 6, 5))}
TILE_SHAPES = {"D2Q9": ((32, 32, 1), (16, 16, 1)), "D3Q19": ((16, 16, 8), (8, 8, 4)), "D3Q27": ((16, 8, 16), (4, 8, 8))}


def to_dev(a: np.ndarray) -> torch.Tensor:
    if a.dtype == np.uint16:
        a = a.view(np.int16)
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def to_host(t: torch.Tensor, like: np.ndarray) -> np.ndarray:
    a = t.cpu().numpy()
    return a.view(np.uint16) if like.dtype == np.uint16 else a


def run_both(grid, cfg: LBM_Config, flags, bc, f0, tau: float, steps: int, threads: int | None = None,
             path: int = 0):
    """Runs `steps` steps on the GPU and in the oracle; returns (gpu f, oracle f, gpu bc, oracle bc).
    path: 0 automatic, 1 generic kernel, 2 block-per-tile kernel."""
    solver = Solver(grid, cfg)
    if threads:
        solver.set_block_threads(threads)
    if path:
        solver.set_kernel_path(path)
        assert solver.kernel_path == path
    fa = to_dev(f0)
    bct = to_dev(bc)
    flt = to_dev(flags)
    f, f2, bco = f0.copy(), f0.copy(), bc.copy()
    if cfg.lbm_method == LBM_method.DOUBLE_BUFFER:
        fb = fa.clone()
        for k in range(steps):
            src, dst = (fa, fb) if k % 2 == 0 else (fb, fa)
            solver.double_buffer_step(dst, src, bct, flt, tau)
            oracle.step(cfg, grid, 32, f2, f, bco, flags, tau)
            f, f2 = f2, f
        out = fa if steps % 2 == 0 else fb
    else:
        for k in range(steps):
            even = k % 2 == 0
            solver.esoteric_pull_step(fa, bct, flt, tau, even)
            oracle.step(cfg, grid, 32, f, f, bco, flags, tau, even)
        out = fa
    torch.cuda.synchronize()
    res = to_host(out, f0), f, bct.cpu().numpy(), bco
    solver.close()
    return res


def assert_close(got: np.ndarray, ref: np.ndarray, cfg: LBM_Config, what: str):
    """Bit-exact comparison of population arrays (float32 words or Float16C codes)."""
    word = np.uint16 if got.dtype == np.uint16 else np.uint32
    g, r = got.view(word), np.ascontiguousarray(ref).view(word)
    bad = g != r
    if bad.any():
        gd = oracle.f16c_decode(got) if word == np.uint16 else got
        rd = oracle.f16c_decode(ref) if word == np.uint16 else ref
        err = float(np.abs(gd.astype(np.float64) - rd).max())
        raise AssertionError(f"{what}: {int(bad.sum())} of {bad.size} words differ (max |df| = {err:.3e})")


CASES = list(itertools.product(["D2Q9", "D3Q19", "D3Q27"], ["db", "eso"], ["fp32", "f16c"],
                               ["SRT", "TRT", "KBC", "RLBM"], [False, True], ["mixed", "ldc"], ["generic", "tile"]))


@pytest.mark.parametrize("lat,meth,store,coll,les,case,kernel", CASES,
                         ids=["-".join(map(str, c)) for c in CASES])
def test_step_parity(lat, meth, store, coll, les, case, kernel):
    shape, tile = (SHAPES if kernel == "generic" else TILE_SHAPES)[lat]
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
    got, ref, bc_gpu, bc_ref = run_both(grid, cfg, flags, bc, f0, tau, STEPS, path=1 if kernel == "generic" else 2)
    assert_close(got, ref, cfg, f"{lat}/{meth}/{store}/{coll}/LES={les}/{case}/{kernel}")
    if case == "mixed":
        # captured rho/u written into bc
        assert np.array_equal(bc_gpu.view(np.uint32), bc_ref.view(np.uint32))


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
@pytest.mark.parametrize("tile", ["untiled", (1, 1, 1), "pow2"])
def test_layouts(lat, tile):
    """The same cavity on the untiled column-major, per-cell (AoS) and power-of-two tiles."""
    shape = {"D2Q9": (32, 16, 1), "D3Q19": (16, 8, 8), "D3Q27": (8, 8, 16)}[lat]
    if tile == "pow2":
        tile = {"D2Q9": (16, 8, 1), "D3Q19": (8, 4, 4), "D3Q27": (4, 8, 2)}[lat]
    grid = make_grid(lat, shape, tile)
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER)
    flags, bc = ldc_flags(grid, cfg, 0.1)
    f0 = initial_f(grid, cfg, np.random.default_rng(3))
    got, ref, _, _ = run_both(grid, cfg, flags, bc, f0, 0.7, 8)
    assert_close(got, ref, cfg, f"layout {tile}")


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
@pytest.mark.parametrize("meth", ["db", "eso"])
@pytest.mark.parametrize("f16", [False, True])
def test_tile_kernel_with_clean_tiles(lat, meth, f16):
    """A cavity of 5+ tiles per axis: all-FLUID tiles take the block-per-tile kernel's fast branch,
    wall tiles the flag branch; a periodic all-fluid grid takes only the fast branch."""
    shape, tile = {"D2Q9": ((80, 80, 1), (16, 16, 1)), "D3Q19": ((40, 40, 20), (8, 8, 4)),
                   "D3Q27": ((20, 40, 40), (4, 8, 8))}[lat]
    grid = make_grid(lat, shape, tile)
    m = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    cfg = LBM_Config(m, DDF_shift=f16, use_float16c=f16, LES=True)
    flags, bc = ldc_flags(grid, cfg, 0.1)
    f0 = initial_f(grid, cfg, np.random.default_rng(21))
    got, ref, _, _ = run_both(grid, cfg, flags, bc, f0, 0.7, 4, path=2)
    assert_close(got, ref, cfg, "cavity")
    flags[:] = 0
    got, ref, _, _ = run_both(grid, cfg, flags, bc, f0, 0.7, 4, path=2)
    assert_close(got, ref, cfg, "periodic")


def test_kernel_path_selection():
    assert Solver(make_grid("D3Q19", (16, 16, 8), (8, 8, 4)), LBM_Config()).kernel_path == 2
    assert Solver(make_grid("D3Q19", (18, 12, 10), (6, 4, 5)), LBM_Config()).kernel_path == 1
    s = Solver(make_grid("D3Q19", (16, 16, 16)), LBM_Config())
    assert s.kernel_path == 1
    with pytest.raises(Exception):
        s.set_kernel_path(2)


@pytest.mark.parametrize("threads", [32, 96, 128, 256])
def test_block_sizes(threads):
    grid = make_grid("D3Q19", (16, 16, 8), (8, 8, 4))
    cfg = LBM_Config(LBM_method.ESOTERIC_PULL, DDF_shift=True)
    flags, bc = ldc_flags(grid, cfg, 0.05)
    f0 = initial_f(grid, cfg, np.random.default_rng(5))
    got, ref, _, _ = run_both(grid, cfg, flags, bc, f0, 0.9, 4, threads, path=1)
    assert_close(got, ref, cfg, f"threads={threads}")


def test_periodic_esoteric_equals_double_buffer():
    """On a periodic all-fluid grid the two streaming methods carry the same populations."""
    grid = make_grid("D3Q27", (12, 8, 8), (4, 4, 4))
    rng = np.random.default_rng(11)
    db = LBM_Config(LBM_method.DOUBLE_BUFFER, collision_op="TRT")
    es = LBM_Config(LBM_method.ESOTERIC_PULL, collision_op="TRT")
    flags = np.zeros(grid.num_points, np.uint8)
    bc = np.zeros(grid.num_points * 4, np.float32)
    u = rng.uniform(-0.03, 0.03, (3,) + grid.shape)
    fdb = np.zeros(grid.num_points * 27, np.float32)
    fes = np.zeros_like(fdb)
    oracle.init(db, grid, 32, fdb, 1.0, 0.8, u)
    oracle.init(es, grid, 32, fes, 1.0, 0.8, u)
    g_db, _, _, _ = run_both(grid, db, flags, bc, fdb, 0.8, 4)
    g_es, _, _, _ = run_both(grid, es, flags, bc, fes, 0.8, 4)
    a = oracle.gather(db, grid, 32, g_db)
    b = oracle.gather(es, grid, 32, g_es, after_odd=True)
    assert np.array_equal(a, b)
