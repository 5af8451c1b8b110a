"""The benchmark configurations at their full size, 256^3, checked bit for bit against the oracle
through the finite propagation speed of the step.

A step reads populations, flags and boundary values of cells at most one cell away, so after k
steps the state of a cell depends only on the initial state, flags and boundary values within k
cells of it.  The 256^3 grid is set up so that a 64^3 corner region (whole 8 x 8 x 4 tiles) holds
the initial state, flags and boundary values of a 64^3 grid that the oracle runs in seconds:
the lid corner (x < 64, y >= 192, z < 64, walls -X, +Y, -Z) of the lid-driven cube, or the
corner x, y, z < 64 of the periodic box.  Every cell of the region at least k + 1 cells away from
the faces where the two grids differ (the small cavity's walls +X, -Y, +Z, or the small box's
periodic wrap) must then hold the oracle's words exactly: float32 words or Float16C codes, as in
the 64^3 parity tests.  The rest of the 256^3 grid starts at rest and is stepped as well.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from mojo_lbm_gb300 import LBM_Config, LBM_method
from mojo_lbm_gb300.solver import Solver
from tests.lbm_cases import initial_f, ldc_flags, make_grid
from tests.test_gpu_step import to_dev

pytestmark = pytest.mark.gpu

BIG, SMALL, TILE, STEPS = 256, 64, (8, 8, 4), 8

# name: lattice, method, collision, LES, Float16C + DDF, tau, cavity (else periodic)
CASES = {
    "ldc_d3q19_fp32": ("D3Q19", "db", "SRT", False, False, 1.265, True),
    "ldc_d3q19_f16c": ("D3Q19", "db", "SRT", False, True, 1.265, True),
    "ldc_d3q27_kbc_les_f16c_eso": ("D3Q27", "eso", "KBC", True, True, 3.0 * 0.1 * 255 / 1e4 + 0.5, True),
    "periodic_d3q19_les_fp32": ("D3Q19", "db", "SRT", True, False, 0.50382, False),
}


def tiles_view(a, n: int, comps: int):
    """[tile z, tile y, tile x, component, z, y, x] view of a tiled array (lx + tx (ly + ty (lz + tz
    (comp + comps tile))), tiles x-fastest) of an n^3 grid with 8 x 8 x 4 tiles."""
    tx, ty, tz = TILE
    return a.reshape(n // tz, n // ty, n // tx, comps, tz, ty, tx)


def cells(v: np.ndarray) -> np.ndarray:
    """[x, y, z, comp] array of a tiles_view of the whole 64^3 region."""
    ntz, nty, ntx, c, tz, ty, tx = v.shape
    return v.transpose(2, 6, 1, 5, 0, 4, 3).reshape(ntx * tx, nty * ty, ntz * tz, c)


@pytest.mark.parametrize("name", list(CASES))
def test_full_size_region_matches_oracle(name):
    lat, meth, coll, les, f16, tau, cavity = CASES[name]
    method = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    cfg = LBM_Config(method, collision_op=coll, LES=les, DDF_shift=f16, use_float16c=f16)
    small = make_grid(lat, (SMALL,) * 3, TILE)
    big = make_grid(lat, (BIG,) * 3, TILE)
    Q, K = small.Q, small.D + 1
    if cavity:
        fl_s, bc_s = ldc_flags(small, cfg, 0.1)
        fl_b, bc_b = ldc_flags(big, cfg, 0.1)
    else:
        fl_s, bc_s = np.zeros(small.num_points, np.uint8), np.zeros(small.num_points * K, np.float32)
        fl_b, bc_b = np.zeros(big.num_points, np.uint8), np.zeros(big.num_points * K, np.float32)
    f0 = initial_f(small, cfg, np.random.default_rng(BIG + Q), tau=tau)

    # the region's tiles in the big grid: y tiles from 192 / 8 = 24 for the lid corner
    ty0 = (BIG - SMALL) // TILE[1] if cavity else 0
    reg = (slice(0, SMALL // TILE[2]), slice(ty0, ty0 + SMALL // TILE[1]), slice(0, SMALL // TILE[0]))
    if cavity:
        # the region's flags and boundary values are the small cavity's, apart from its own walls
        # +X, -Y, +Z, which the compared cells do not reach
        sm_fl = cells(tiles_view(fl_s, SMALL, 1))
        bg_fl = cells(tiles_view(fl_b, BIG, 1)[reg])
        assert np.array_equal(sm_fl[: SMALL - 1, 1:, : SMALL - 1], bg_fl[: SMALL - 1, 1:, : SMALL - 1])
        sm_bc = cells(tiles_view(bc_s, SMALL, K))
        bg_bc = cells(tiles_view(bc_b, BIG, K)[reg])
        assert np.array_equal(sm_bc[: SMALL - 1, 1:, : SMALL - 1].view(np.uint32),
                              bg_bc[: SMALL - 1, 1:, : SMALL - 1].view(np.uint32))

    solver = Solver(big, cfg)
    fa = torch.empty(big.num_points * Q, dtype=torch.int16 if f16 else torch.float32, device="cuda")
    solver.init_equilibrium(fa)
    tiles_view(fa, BIG, Q)[reg] = tiles_view(to_dev(f0), SMALL, Q)
    fb = fa.clone() if meth == "db" else None
    bct, flt = to_dev(bc_b), to_dev(fl_b)
    solver.run(fa, fb, bct, flt, tau, STEPS, 0)
    got = tiles_view(fa, BIG, Q)[reg].cpu().numpy()
    solver.close()
    del fa, fb, bct, flt
    torch.cuda.empty_cache()

    f, f2 = f0.copy(), f0.copy()
    for k in range(STEPS):
        if meth == "db":
            oracle.step(cfg, small, 32, f2, f, bc_s, fl_s, tau)
            f, f2 = f2, f
        else:
            oracle.step(cfg, small, 32, f, f, bc_s, fl_s, tau, k % 2 == 0)

    word = np.uint16 if f16 else np.uint32
    g = cells(got.view(word))
    w = cells(tiles_view(f, SMALL, Q).view(word))
    k1 = STEPS + 1
    if cavity:
        keep = (slice(0, SMALL - k1), slice(k1, SMALL), slice(0, SMALL - k1))
    else:
        keep = (slice(k1 - 1, SMALL - k1 + 1),) * 3
    g, w = g[keep], w[keep]
    bad = g != w
    if bad.any():
        gd = oracle.f16c_decode(g) if f16 else g.view(np.float32)
        wd = oracle.f16c_decode(w) if f16 else w.view(np.float32)
        err = float(np.abs(gd.astype(np.float64) - wd).max())
        raise AssertionError(f"{name}: {int(bad.sum())} of {bad.size} words differ (max |df| = {err:.3e})")
    # the compared cells moved away from their initial state
    f0c = cells(tiles_view(f0, SMALL, Q).view(word))[keep]
    assert (w != f0c).mean() > 0.5
