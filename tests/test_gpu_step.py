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
import json
import zlib
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle
from mojo_lbm_gb300 import Flags, LBM_Config, LBM_method
from mojo_lbm_gb300.solver import Solver
from tests.lbm_cases import digest, initial_f, ldc_flags, make_grid, mixed_flags, step_case

pytestmark = pytest.mark.gpu

STEPS = 6
GOLDENS = json.loads((Path(__file__).with_name("golden") / "oracle_goldens.json").read_text())
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
    # the recipe of the oracle's goldens (tests/golden/make_oracle_goldens.py)
    grid, cfg, flags, bc, f0, tau = step_case(lat, meth, store, coll, les, case, shape, tile)
    got, ref, bc_gpu, bc_ref = run_both(grid, cfg, flags, bc, f0, tau, STEPS, path=1 if kernel == "generic" else 2)
    assert_close(got, ref, cfg, f"{lat}/{meth}/{store}/{coll}/LES={les}/{case}/{kernel}")
    if case == "mixed":
        # captured rho/u written into bc
        assert np.array_equal(bc_gpu.view(np.uint32), bc_ref.view(np.uint32))
    if kernel == "generic":
        # the committed digest of this case's output (tests/golden/oracle_goldens.json)
        assert GOLDENS["steps"] == STEPS and GOLDENS["shapes"][lat] == [list(shape), list(tile)]
        want = GOLDENS["cases"]["-".join(map(str, (lat, meth, store, coll, les, case)))]["outputs"]
        assert digest(got, bc_gpu) == want


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


# Tile shapes whose warps own boxes of different shape (x rows of 32, slabs, columns): 256 x 1 and
# 32 x 8 -> 32 x 1 boxes; 16 x 16 -> 16 x 2; 4 x 64 -> 4 x 8; 1 x 256 -> 1 x 32; 8 x 8 x 4 -> 8 x 4 x 1;
# 2 x 4 x 32 -> 2 x 4 x 4; 1 x 16 x 16 -> 1 x 16 x 2; 1 x 1 x 256 -> 1 x 1 x 32.
WARP_BOX_TILES = {"D2Q9": ((256, 256, 1), [(256, 1, 1), (32, 8, 1), (16, 16, 1), (4, 64, 1), (1, 256, 1)]),
                  "D3Q19": ((64, 32, 32), [(32, 8, 1), (8, 8, 4), (2, 4, 32), (1, 16, 16), (64, 2, 2)]),
                  "D3Q27": ((16, 16, 256), [(4, 8, 8), (16, 4, 4), (1, 1, 256)])}
WARP_BOX_CASES = [(lat, t, meth, f16) for lat, (_, ts) in WARP_BOX_TILES.items() for t in ts
                  for meth in ("db", "eso") for f16 in (False, True)]


@pytest.mark.parametrize("lat,tile,meth,f16", WARP_BOX_CASES,
                         ids=[f"{c[0]}-{'x'.join(map(str, c[1]))}-{c[2]}-{'f16c' if c[3] else 'fp32'}"
                              for c in WARP_BOX_CASES])
def test_sparse_flags_warp_masks(lat, tile, meth, f16):
    """Isolated flags of every kind in an otherwise plain-FLUID periodic grid: only the warps whose
    32 cells or 1-cell halo (across warp-box, tile and periodic edges) hold one take the flag
    branch of the block-per-tile kernel, the rest the fast branch; bit-exact against the oracle."""
    shape = WARP_BOX_TILES[lat][0]
    grid = make_grid(lat, shape, tile)
    rng = np.random.default_rng(zlib.crc32(f"sparse/{lat}/{tile}/{meth}/{f16}".encode()))
    m = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    cfg = LBM_Config(m, BCs={Flags.EQUILIBRIUM}, DDF_shift=f16, use_float16c=f16, capture_density=True,
                     capture_velocity=True)
    flags, bc = mixed_flags(grid, rng)
    flags[rng.random(flags.size) >= 0.004] = 0
    f0 = initial_f(grid, cfg, rng)
    got, ref, bc_gpu, bc_ref = run_both(grid, cfg, flags, bc, f0, 0.8, 4, path=2)
    assert_close(got, ref, cfg, f"sparse flags, tile {tile}")
    assert np.array_equal(bc_gpu.view(np.uint32), bc_ref.view(np.uint32))


@pytest.mark.parametrize("f16", [False, True])
def test_flags_changing_between_steps(f16):
    """One handle stepped with a flag field that changes between calls (rewritten in place, and a
    second buffer), by single steps and by graph-replayed runs: the block-per-tile kernel's warp
    masks follow every change; bit-exact against the oracle."""
    grid = make_grid("D3Q19", (32, 32, 16), (8, 8, 4))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, BCs={Flags.EQUILIBRIUM}, DDF_shift=f16, use_float16c=f16,
                     capture_density=True, capture_velocity=True)
    rng = np.random.default_rng(77)
    fl_a, bc = mixed_flags(grid, rng)
    fl_a[rng.random(fl_a.size) >= 0.01] = 0
    # fixed boundary values everywhere (no free NaN components): a cell that is EQUILIBRIUM in one
    # field is a wall in another, and a wall's velocity and density must be numbers
    comp = (np.arange(bc.size) // grid.layouts.T) % (grid.D + 1)
    bc[np.isnan(bc)] = np.where(comp[np.isnan(bc)] == grid.D, 1.0, 0.0)
    fl_b, _ = ldc_flags(grid, cfg, 0.1)
    fl_c = np.zeros_like(fl_a)
    f0 = initial_f(grid, cfg, rng)
    solver = Solver(grid, cfg)
    assert solver.kernel_path in (2, 3)
    fa, fb, bct = to_dev(f0), to_dev(f0), to_dev(bc)
    flt, flt2 = to_dev(fl_a), to_dev(fl_b)
    f, f2, bco = f0.copy(), f0.copy(), bc.copy()
    k = 0
    # (flag field, buffer: 0 = the first buffer, rewritten in place with the field; 1 = a second
    # buffer holding fl_b, steps, by graph-replayed run)
    plan = [(fl_a, 0, 2, False), (fl_b, 1, 3, False), (fl_a, 0, 1, False), (fl_c, 0, 2, False),
            (fl_b, 1, 64, True), (fl_a, 0, 64, True), (fl_b, 0, 1, False), (fl_b, 1, 1, False)]
    for host, which, n, by_run in plan:
        if which == 0:
            flt.copy_(to_dev(host))
        dev = flt if which == 0 else flt2
        if by_run:
            solver.run(fa, fb, bct, dev, 0.8, n, k)
        else:
            for j in range(n):
                src, dst = (fa, fb) if (k + j) % 2 == 0 else (fb, fa)
                solver.double_buffer_step(dst, src, bct, dev, 0.8)
        for _ in range(n):
            oracle.step(cfg, grid, 32, f2, f, bco, host, 0.8)
            f, f2 = f2, f
        k += n
    torch.cuda.synchronize()
    got = to_host(fa if k % 2 == 0 else fb, f0)
    solver.close()
    assert_close(got, f, cfg, "changing flags")
    assert np.array_equal(bct.cpu().numpy().view(np.uint32), bco.view(np.uint32))


@pytest.mark.parametrize("f16", [False, True])
@pytest.mark.parametrize("kernel", ["generic", "tile"])
@pytest.mark.parametrize("coll,les", [("SRT", False), ("SRT", True), ("KBC", True), ("KBC", False)])
def test_fluid_at_rest(f16, kernel, coll, les):
    """A periodic box at rest (zero momentum in every cell: the velocity's signed zeros, KBC's zero
    entropic terms and the zero strain norm are taken without dividing or a square root), then one
    cell disturbed: bit-exact against the oracle."""
    shape, tile = ((18, 12, 10), (6, 4, 5)) if kernel == "generic" else ((16, 16, 8), (8, 8, 4))
    grid = make_grid("D3Q19", shape, tile)
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, collision_op=coll, LES=les, DDF_shift=f16, use_float16c=f16,
                     include_moving_boundary=False)
    flags = np.zeros(grid.num_points, np.uint8)
    bc = np.zeros(grid.num_points * 4, np.float32)
    f0 = initial_f(grid, cfg, None)
    got, ref, _, _ = run_both(grid, cfg, flags, bc, f0, 0.884, 4, path=1 if kernel == "generic" else 2)
    assert_close(got, ref, cfg, "at rest")
    f1 = f0.copy()
    f1[grid.Q * 0 + 5] = oracle.f16c_encode(np.array([1e-3], np.float32))[0] if f16 else f1[5] + np.float32(1e-3)
    got, ref, _, _ = run_both(grid, cfg, flags, bc, f1, 0.884, 6, path=1 if kernel == "generic" else 2)
    assert_close(got, ref, cfg, "one cell disturbed")


def test_kernel_path_selection():
    assert Solver(make_grid("D3Q19", (128, 128, 64), (8, 8, 4)), LBM_Config()).kernel_path == 3  # cell pairs
    assert Solver(make_grid("D3Q19", (16, 16, 8), (8, 8, 4)), LBM_Config()).kernel_path == 2  # few tiles
    assert Solver(make_grid("D3Q19", (16, 16, 8), (8, 8, 4)), LBM_Config(collision_op="KBC")).kernel_path == 2
    assert Solver(make_grid("D3Q19", (16, 16, 8), (8, 8, 4)),
                  LBM_Config(LBM_method.ESOTERIC_PULL)).kernel_path == 2
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
