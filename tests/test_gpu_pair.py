"""The cell-pair block-per-tile kernel (kernel path 3: one thread per two cells along x, word-wide
population accesses) against the float32 CPU oracle and against the per-cell block-per-tile
kernel.

Exact arithmetic: no tolerance.  The pair kernel runs the per-cell code of the block-per-tile
kernel on each of its two cells, so populations (float32 words or Float16C codes) and captured bc
values equal the oracle's bit for bit.  Fast arithmetic: the same per-cell code as the fast
block-per-tile kernel, whose tolerance against the oracle tests/test_gpu_fast.py states; here the
two kernels are compared with each other, word for word.
"""
from __future__ import annotations

import itertools
import zlib

import numpy as np
import pytest
import torch

from mojo_lbm_gb300 import Flags, LBM_Config, LBM_method
from mojo_lbm_gb300.solver import Solver
from tests.lbm_cases import initial_f, ldc_flags, make_grid, mixed_flags, step_case
from tests.test_gpu_step import assert_close, run_both, to_dev, to_host

pytestmark = pytest.mark.gpu

TILE_SHAPES = {"D2Q9": ((32, 32, 1), (16, 16, 1)), "D3Q19": ((16, 16, 8), (8, 8, 4)), "D3Q27": ((16, 8, 16), (4, 8, 8))}
CASES = list(itertools.product(["D2Q9", "D3Q19", "D3Q27"], ["fp32", "f16c"], ["SRT", "TRT", "KBC", "RLBM"],
                               [False, True], ["mixed", "ldc"]))


@pytest.mark.parametrize("lat,store,coll,les,case", CASES, ids=["-".join(map(str, c)) for c in CASES])
def test_pair_step_parity(lat, store, coll, les, case):
    shape, tile = TILE_SHAPES[lat]
    grid, cfg, flags, bc, f0, tau = step_case(lat, "db", store, coll, les, case, shape, tile)
    got, ref, bc_gpu, bc_ref = run_both(grid, cfg, flags, bc, f0, tau, 6, path=3)
    assert_close(got, ref, cfg, f"pair {lat}/{store}/{coll}/LES={les}/{case}")
    if case == "mixed":
        assert np.array_equal(bc_gpu.view(np.uint32), bc_ref.view(np.uint32))


# tiles with tx >= 2 whose warps own boxes of different shapes (the pair kernel's warp owns two)
PAIR_TILES = {"D2Q9": ((256, 256, 1), [(256, 1, 1), (32, 8, 1), (16, 16, 1), (4, 64, 1), (2, 128, 1)]),
              "D3Q19": ((64, 32, 32), [(32, 8, 1), (8, 8, 4), (2, 4, 32), (64, 2, 2)]),
              "D3Q27": ((16, 16, 256), [(4, 8, 8), (16, 4, 4), (2, 2, 64)])}
PAIR_TILE_CASES = [(lat, t, f16) for lat, (_, ts) in PAIR_TILES.items() for t in ts for f16 in (False, True)]


@pytest.mark.parametrize("lat,tile,f16", PAIR_TILE_CASES,
                         ids=[f"{c[0]}-{'x'.join(map(str, c[1]))}-{'f16c' if c[2] else 'fp32'}" for c in PAIR_TILE_CASES])
def test_pair_sparse_flags(lat, tile, f16):
    """Isolated flags of every kind in a periodic grid: pairs whose box is flagged next to pairs
    whose box is clear in the same warp, a SOLID or EXCLUDE cell beside an active one (half-pair
    stores), tile-edge x neighbours (tx = 2: every pair touches both x edges)."""
    grid = make_grid(lat, PAIR_TILES[lat][0], tile)
    rng = np.random.default_rng(zlib.crc32(f"pair/{lat}/{tile}/{f16}".encode()))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, BCs={Flags.EQUILIBRIUM}, DDF_shift=f16, use_float16c=f16,
                     capture_density=True, capture_velocity=True)
    flags, bc = mixed_flags(grid, rng)
    flags[rng.random(flags.size) >= 0.004] = 0
    f0 = initial_f(grid, cfg, rng)
    got, ref, bc_gpu, bc_ref = run_both(grid, cfg, flags, bc, f0, 0.8, 4, path=3)
    assert_close(got, ref, cfg, f"pair sparse flags, tile {tile}")
    assert np.array_equal(bc_gpu.view(np.uint32), bc_ref.view(np.uint32))


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
@pytest.mark.parametrize("f16", [False, True])
def test_pair_cavity_and_periodic(lat, f16):
    shape, tile = {"D2Q9": ((80, 80, 1), (16, 16, 1)), "D3Q19": ((40, 40, 20), (8, 8, 4)),
                   "D3Q27": ((20, 40, 40), (4, 8, 8))}[lat]
    grid = make_grid(lat, shape, tile)
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, DDF_shift=f16, use_float16c=f16, LES=True)
    flags, bc = ldc_flags(grid, cfg, 0.1)
    f0 = initial_f(grid, cfg, np.random.default_rng(21))
    got, ref, _, _ = run_both(grid, cfg, flags, bc, f0, 0.7, 4, path=3)
    assert_close(got, ref, cfg, "cavity")
    flags[:] = 0
    got, ref, _, _ = run_both(grid, cfg, flags, bc, f0, 0.7, 4, path=3)
    assert_close(got, ref, cfg, "periodic")


def _run(grid, cfg, flags, bc, f0, tau, steps, path, offset=0):
    """`steps` graph-replayed steps (lbm_run) on the kernel path; offset > 0 places the lattices
    `offset` elements into larger buffers (misaligned for the pair kernel's words)."""
    s = Solver(grid, cfg)
    s.set_kernel_path(path)
    n = f0.size
    base_a, base_b = to_dev(np.concatenate([f0[:offset], f0])), to_dev(np.concatenate([f0[:offset], f0]))
    fa, fb = base_a[offset:offset + n], base_b[offset:offset + n]
    bct, flt = to_dev(bc), to_dev(flags)
    s.run(fa, fb, bct, flt, tau, steps, 0)
    torch.cuda.synchronize()
    out = to_host(fa if steps % 2 == 0 else fb, f0)
    s.close()
    return out, bct.cpu().numpy()


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
@pytest.mark.parametrize("store", ["fp32", "f16c"])
@pytest.mark.parametrize("coll,les", [("SRT", False), ("SRT", True), ("TRT", False), ("KBC", True), ("RLBM", False)])
def test_pair_fast_equals_tile_fast(lat, store, coll, les):
    """The fast arithmetic: the pair kernel's populations and captures equal the per-cell
    block-per-tile kernel's word for word (same per-cell code), over 66 graph-replayed steps."""
    shape, tile = TILE_SHAPES[lat]
    grid, cfg, flags, bc, f0, tau = step_case(lat, "db", store, coll, les, "mixed", shape, tile)
    cfg.arithmetic = "fast"
    a, bca = _run(grid, cfg, flags, bc, f0, tau, 66, 2)
    b, bcb = _run(grid, cfg, flags, bc, f0, tau, 66, 3)
    word = np.uint16 if a.dtype == np.uint16 else np.uint32
    assert np.array_equal(a.view(word), b.view(word))
    assert np.array_equal(bca.view(np.uint32), bcb.view(np.uint32))


@pytest.mark.parametrize("store", ["fp32", "f16c"])
def test_pair_misaligned_buffers_fall_back(store):
    """Population buffers that are not 8-byte aligned run the per-cell kernel: same results."""
    shape, tile = TILE_SHAPES["D3Q19"]
    grid, cfg, flags, bc, f0, tau = step_case("D3Q19", "db", store, "SRT", False, "ldc", shape, tile)
    a, _ = _run(grid, cfg, flags, bc, f0, tau, 64, 3)
    b, _ = _run(grid, cfg, flags, bc, f0, tau, 64, 3, offset=1)
    word = np.uint16 if a.dtype == np.uint16 else np.uint32
    assert np.array_equal(a.view(word), b.view(word))


def test_pair_path_selection():
    s = Solver(make_grid("D3Q19", (16, 16, 8), (8, 8, 4)), LBM_Config())
    assert s.kernel_path == 2  # 8 tiles: the automatic choice is the per-cell kernel
    s.set_kernel_path(3)
    assert s.kernel_path == 3
    s.close()
    s = Solver(make_grid("D3Q19", (128, 128, 64), (8, 8, 4)), LBM_Config())
    s.set_kernel_path(3)
    assert s.kernel_path == 3
    s.set_kernel_path(2)
    assert s.kernel_path == 2
    s.set_kernel_path(0)
    assert s.kernel_path == 3  # the automatic choice for D3Q19 SRT on 4096 tiles
    s.close()
    s = Solver(make_grid("D2Q9", (1024, 608, 1), (16, 16, 1)), LBM_Config())
    assert s.kernel_path == 3  # 2432 tiles, the smallest grid the automatic choice gives cell pairs
    s.close()
    s = Solver(make_grid("D2Q9", (1024, 592, 1), (16, 16, 1)), LBM_Config())
    assert s.kernel_path == 2  # 2368 tiles
    s.close()
    for grid, cfg in ((make_grid("D3Q19", (16, 16, 8), (8, 8, 4)), LBM_Config(LBM_method.ESOTERIC_PULL)),
                      (make_grid("D3Q19", (16, 64, 8), (1, 64, 4)), LBM_Config()),
                      (make_grid("D3Q19", (18, 12, 10), (6, 4, 5)), LBM_Config())):
        s = Solver(grid, cfg)
        with pytest.raises(Exception):
            s.set_kernel_path(3)
        s.close()
