"""The staged block-per-tile kernel (kernel path 4: persistent CTAs; bulk asynchronous copies stage
each tile's pull neighbourhood in shared memory, double-buffered) against the float32 CPU oracle
and against the per-cell block-per-tile kernel, and its bounded wait.

Exact arithmetic: no tolerance (the staged kernel runs tile_step's per-cell code on values read
from the stage, which equal the pull loads: tests/test_stage_cpu.py).  Fast arithmetic: equal to
the fast block-per-tile kernel word for word.  The wait: with 16 bytes more expected than the copies
deliver, every stage's wait runs out after 0.5 s, the kernel raises its error word and returns, the
host reports LBM_ETIMEOUT, and the handle steps correctly afterwards.
"""
from __future__ import annotations

import itertools
import zlib

import numpy as np
import pytest
import torch

import oracle
from mojo_lbm_gb300 import Flags, LBM_Config, LBM_method, _capi
from mojo_lbm_gb300.solver import Solver
from tests.lbm_cases import initial_f, ldc_flags, make_grid, mixed_flags, step_case
from tests.test_gpu_step import assert_close, run_both, to_dev, to_host

pytestmark = pytest.mark.gpu

# tiles whose rows are 16-byte multiples for both storages (tx >= 8)
SHAPES = {"D2Q9": ((32, 32, 1), (16, 16, 1)), "D3Q19": ((16, 16, 8), (8, 8, 4)), "D3Q27": ((16, 16, 8), (8, 8, 4))}
CASES = list(itertools.product(["D2Q9", "D3Q19", "D3Q27"], ["fp32", "f16c"], ["SRT", "TRT", "KBC", "RLBM"],
                               [False, True], ["mixed", "ldc"]))


@pytest.mark.parametrize("lat,store,coll,les,case", CASES, ids=["-".join(map(str, c)) for c in CASES])
def test_staged_step_parity(lat, store, coll, les, case):
    shape, tile = SHAPES[lat]
    grid, cfg, flags, bc, f0, tau = step_case(lat, "db", store, coll, les, case, shape, tile)
    got, ref, bc_gpu, bc_ref = run_both(grid, cfg, flags, bc, f0, tau, 6, path=4)
    assert_close(got, ref, cfg, f"staged {lat}/{store}/{coll}/LES={les}/{case}")
    if case == "mixed":
        assert np.array_equal(bc_gpu.view(np.uint32), bc_ref.view(np.uint32))


@pytest.mark.parametrize("lat,shape,tile", [("D3Q19", (128, 64, 64), (8, 8, 4)), ("D3Q19", (64, 64, 64), (16, 4, 4)),
                                            ("D2Q9", (512, 512, 1), (16, 16, 1)), ("D3Q27", (64, 64, 64), (8, 8, 4))])
@pytest.mark.parametrize("f16", [False, True])
def test_staged_persistent_walk(lat, shape, tile, f16):
    """Grids of 1024-4096 tiles: every CTA walks several tiles through both stage buffers (both
    mbarrier phases), on a cavity (walls on five faces, a moving lid) with equilibrium cells."""
    grid = make_grid(lat, shape, tile)
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, BCs={Flags.EQUILIBRIUM}, DDF_shift=f16, use_float16c=f16, LES=True)
    flags, bc = ldc_flags(grid, cfg, 0.1)
    rng = np.random.default_rng(zlib.crc32(f"walk/{lat}/{shape}/{f16}".encode()))
    f0 = initial_f(grid, cfg, rng)
    got, ref, _, _ = run_both(grid, cfg, flags, bc, f0, 0.7, 5, path=4)
    assert_close(got, ref, cfg, f"staged walk {lat} {shape}")


STAGE_TILES = {"D2Q9": ((256, 256, 1), [(256, 1, 1), (32, 8, 1), (16, 16, 1), (8, 32, 1)]),
               "D3Q19": ((64, 32, 32), [(32, 8, 1), (8, 8, 4), (8, 4, 8), (64, 2, 2)]),
               "D3Q27": ((16, 16, 256), [(8, 8, 4), (16, 4, 4), (8, 2, 16)])}
STAGE_TILE_CASES = [(lat, t, f16) for lat, (_, ts) in STAGE_TILES.items() for t in ts for f16 in (False, True)]


@pytest.mark.parametrize("lat,tile,f16", STAGE_TILE_CASES,
                         ids=[f"{c[0]}-{'x'.join(map(str, c[1]))}-{'f16c' if c[2] else 'fp32'}" for c in STAGE_TILE_CASES])
def test_staged_sparse_flags(lat, tile, f16):
    """Isolated flags of every kind in a periodic grid, several tile shapes: the staged values
    with the warp masks, bounce-back reloads, equilibrium cells and captures."""
    grid = make_grid(lat, STAGE_TILES[lat][0], tile)
    rng = np.random.default_rng(zlib.crc32(f"stage/{lat}/{tile}/{f16}".encode()))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, BCs={Flags.EQUILIBRIUM}, DDF_shift=f16, use_float16c=f16,
                     capture_density=True, capture_velocity=True)
    flags, bc = mixed_flags(grid, rng)
    flags[rng.random(flags.size) >= 0.004] = 0
    f0 = initial_f(grid, cfg, rng)
    got, ref, bc_gpu, bc_ref = run_both(grid, cfg, flags, bc, f0, 0.8, 4, path=4)
    assert_close(got, ref, cfg, f"staged sparse flags, tile {tile}")
    assert np.array_equal(bc_gpu.view(np.uint32), bc_ref.view(np.uint32))


def _run(grid, cfg, flags, bc, f0, tau, steps, path, offset=0):
    s = Solver(grid, cfg)
    s.set_kernel_path(path)
    n = f0.size
    base_a, base_b = to_dev(np.concatenate([f0[:offset], f0])), to_dev(np.concatenate([f0[:offset], f0]))
    fa, fb = base_a[offset:offset + n], base_b[offset:offset + n]
    bct, flt = to_dev(bc), to_dev(flags)
    s.run(fa, fb, bct, flt, tau, steps, 0)
    s.device_status()
    out = to_host(fa if steps % 2 == 0 else fb, f0)
    s.close()
    return out, bct.cpu().numpy()


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
@pytest.mark.parametrize("store", ["fp32", "f16c"])
@pytest.mark.parametrize("coll,les", [("SRT", False), ("SRT", True), ("TRT", False), ("KBC", True), ("RLBM", False)])
def test_staged_fast_equals_tile_fast(lat, store, coll, les):
    shape, tile = SHAPES[lat]
    grid, cfg, flags, bc, f0, tau = step_case(lat, "db", store, coll, les, "mixed", shape, tile)
    cfg.arithmetic = "fast"
    a, bca = _run(grid, cfg, flags, bc, f0, tau, 66, 2)
    b, bcb = _run(grid, cfg, flags, bc, f0, tau, 66, 4)
    word = np.uint16 if a.dtype == np.uint16 else np.uint32
    assert np.array_equal(a.view(word), b.view(word))
    assert np.array_equal(bca.view(np.uint32), bcb.view(np.uint32))


@pytest.mark.parametrize("store", ["fp32", "f16c"])
def test_staged_misaligned_buffers_fall_back(store):
    """Population buffers off a 16-byte boundary run the per-cell kernel: same populations."""
    grid, cfg, flags, bc, f0, tau = step_case("D3Q19", "db", store, "SRT", False, "ldc", *SHAPES["D3Q19"])
    a, _ = _run(grid, cfg, flags, bc, f0, tau, 64, 4)
    b, _ = _run(grid, cfg, flags, bc, f0, tau, 64, 4, offset=4)
    word = np.uint16 if a.dtype == np.uint16 else np.uint32
    assert np.array_equal(a.view(word), b.view(word))


def test_staged_wait_runs_out():
    grid, cfg, flags, bc, f0, tau = step_case("D3Q19", "db", "f16c", "SRT", False, "ldc", *SHAPES["D3Q19"])
    s = Solver(grid, cfg)
    s.set_kernel_path(4)
    fa, fb, bct, flt = to_dev(f0), to_dev(f0), to_dev(bc), to_dev(flags)
    lib = _capi.lib()
    _capi.check(lib.lbm_debug_stage_extra_bytes(s._h, 16))
    s.double_buffer_step(fb, fa, bct, flt, tau)
    with pytest.raises(Exception, match="LBM_ETIMEOUT|ran out"):
        s.device_status()
    s.device_status()  # cleared
    _capi.check(lib.lbm_debug_stage_extra_bytes(s._h, 0))
    ref = f0.copy()
    out = f0.copy()
    oracle.step(cfg, grid, 32, out, ref, bc.copy(), flags, tau)
    s.double_buffer_step(fb, fa, bct, flt, tau)
    s.device_status()
    assert_close(to_host(fb, f0), out, cfg, "after the timeout")
    s.close()


def test_staged_path_selection():
    s = Solver(make_grid("D3Q19", (16, 16, 8), (8, 8, 4)), LBM_Config(use_float16c=True, DDF_shift=True))
    s.set_kernel_path(4)
    assert s.kernel_path == 4
    s.close()
    for grid, cfg in ((make_grid("D3Q19", (16, 16, 8), (8, 8, 4)), LBM_Config(LBM_method.ESOTERIC_PULL)),
                      (make_grid("D3Q19", (16, 64, 8), (4, 16, 4)), LBM_Config(use_float16c=True, DDF_shift=True)),
                      (make_grid("D3Q19", (18, 12, 10), (6, 4, 5)), LBM_Config())):
        s = Solver(grid, cfg)
        with pytest.raises(Exception):
            s.set_kernel_path(4)
        s.close()
