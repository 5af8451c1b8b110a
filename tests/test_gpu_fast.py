"""Parity of the fast-arithmetic step (LBM_ARITH_FAST) with the float32 CPU oracle, to a stated
tolerance.

The fast build rearranges the reference's operators for fused multiply-add (moments from opposite
pairs, one equilibrium per pair, approximate reciprocals; Float16C codes in a scaled form), so it
is not bit-identical to the reference's operation order.  Each step is checked on its own: the
oracle steps from the GPU's previous state, so the errors measured are those of one step, not an
accumulation.  Tolerances, per step:
  float32 populations   |f_fast - f_oracle| <= 1e-6 + 2e-6 |f_oracle|
  Float16C populations  the float32 tolerance plus one unit in the code's last place, on the
                        decoded values: 1e-6 + (2e-6 + 2^-10) |f| (2^-10 |f| bounds one ulp of the
                        11-bit mantissa).  The float32 part matters where |f| is small (DDF-shifted
                        populations near 1e-4, whose code ulp is 3e-8): there a float32 difference
                        of 1e-7, which KBC's entropic ratio <ds,dh>/<dh,dh> reaches under any
                        reordering of its sums, is several code ulps.
  captured rho / u      |d| <= 2e-6 + 2e-6 |value|
Every lattice x streaming method x storage x collision operator x LES, on the two seeded cases of
the exact step-parity tests ('mixed': every boundary branch, capture bits, EXCLUDE, free NaN bc
components; 'ldc': closed cavity with a moving lid), on the block-per-tile kernel.
"""
from __future__ import annotations

import itertools

import numpy as np
import pytest
import torch

import oracle
from mojo_lbm_gb300 import LBM_Config, LBM_method
from mojo_lbm_gb300.solver import Solver
from tests.lbm_cases import fluid_mask_pop, initial_f, ldc_flags, make_grid, step_case

pytestmark = pytest.mark.gpu

TILE_SHAPES = {"D2Q9": ((32, 32, 1), (16, 16, 1)), "D3Q19": ((16, 16, 8), (8, 8, 4)), "D3Q27": ((16, 8, 16), (4, 8, 8))}
F32_ABS, F32_REL = 1e-6, 2e-6


def _fast(cfg: LBM_Config) -> LBM_Config:
    cfg.arithmetic = "fast"
    return cfg


def to_dev(a: np.ndarray) -> torch.Tensor:
    if a.dtype == np.uint16:
        a = a.view(np.int16)
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def to_host(t: torch.Tensor, like: np.ndarray) -> np.ndarray:
    a = t.cpu().numpy()
    return a.view(np.uint16) if like.dtype == np.uint16 else a


def check_pop(got: np.ndarray, ref: np.ndarray, mask: np.ndarray, what: str):
    """The per-step tolerance of the fast build on the populations selected by mask."""
    if got.dtype == np.uint16:
        g = oracle.f16c_decode(got[mask]).astype(np.float64)
        r = oracle.f16c_decode(ref[mask]).astype(np.float64)
        tol = F32_ABS + (F32_REL + 2.0 ** -10) * np.abs(r)
    else:
        g, r = got[mask].astype(np.float64), ref[mask].astype(np.float64)
        tol = F32_ABS + F32_REL * np.abs(r)
    both_nan = np.isnan(g) & np.isnan(r)
    err = np.where(both_nan, 0.0, np.abs(g - r))
    bad = ~(err <= tol)
    if bad.any():
        i = int(np.argmax(np.where(bad, err - tol, -np.inf)))
        raise AssertionError(f"{what}: {int(bad.sum())} of {bad.size} values beyond the tolerance "
                             f"(worst |df| = {err[i]:.3e} at |f| = {abs(r[i]):.3e}, tol {tol[i]:.3e})")
    return float((err / tol).max()) if err.size else 0.0


def step_pairs(grid, cfg: LBM_Config, flags, bc, f0, tau: float, steps: int):
    """Runs `steps` fast GPU steps; after each, the oracle's step from the same input.  Yields
    (k, gpu output, oracle output, gpu bc, oracle bc)."""
    solver = Solver(grid, cfg)
    assert solver.kernel_path in (2, 3), "the fast arithmetic runs in the block-per-tile kernels"
    fa = to_dev(f0)
    bct = to_dev(bc)
    flt = to_dev(flags)
    db = cfg.lbm_method == LBM_method.DOUBLE_BUFFER
    fb = fa.clone() if db else fa
    try:
        for k in range(steps):
            src, dst = (fa, fb) if k % 2 == 0 else (fb, fa)
            x = to_host(src, f0)
            bco = bct.cpu().numpy()
            if db:
                y = to_host(dst, f0)  # cells the step does not write (SOLID, EXCLUDE) keep these
                solver.double_buffer_step(dst, src, bct, flt, tau)
                oracle.step(cfg, grid, 32, y, x, bco, flags, tau)
            else:
                solver.esoteric_pull_step(fa, bct, flt, tau, k % 2 == 0)
                y = x
                oracle.step(cfg, grid, 32, y, y, bco, flags, tau, k % 2 == 0)
            torch.cuda.synchronize()
            yield k, to_host(dst, f0), y, bct.cpu().numpy(), bco
    finally:
        solver.close()


CASES = list(itertools.product(["D2Q9", "D3Q19", "D3Q27"], ["db", "eso"], ["fp32", "f16c"],
                               ["SRT", "TRT", "KBC", "RLBM"], [False, True], ["mixed", "ldc"]))


@pytest.mark.parametrize("lat,meth,store,coll,les,case", CASES, ids=["-".join(map(str, c)) for c in CASES])
def test_fast_step_tolerance(lat, meth, store, coll, les, case):
    shape, tile = TILE_SHAPES[lat]
    grid, cfg, flags, bc, f0, tau = step_case(lat, meth, store, coll, les, case, shape, tile)
    _fast(cfg)
    mask = np.ones(f0.size, bool)  # every slot: unwritten cells must come through unchanged
    worst = 0.0
    for k, got, ref, bc_gpu, bc_ref in step_pairs(grid, cfg, flags, bc, f0, tau, 4):
        worst = max(worst, check_pop(got, ref, mask, f"{lat}/{meth}/{store}/{coll}/LES={les}/{case} step {k}"))
        if case == "mixed":
            g, r = bc_gpu.astype(np.float64), bc_ref.astype(np.float64)
            ok = (np.isnan(g) & np.isnan(r)) | (np.abs(g - r) <= 2e-6 + 2e-6 * np.abs(r))
            assert ok.all(), f"captured bc step {k}: {int((~ok).sum())} values differ"
    print(f"[fast tolerance] {lat}/{meth}/{store}/{coll}/LES={les}/{case}: worst error / tolerance = {worst:.3f}")


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
@pytest.mark.parametrize("meth", ["db", "eso"])
@pytest.mark.parametrize("f16", [False, True])
@pytest.mark.parametrize("coll", ["SRT", "KBC"])
def test_fast_clean_warps(lat, meth, f16, coll):
    """A cavity of 5+ tiles per axis, so most warps take the kernel's all-fluid branch."""
    shape, tile = {"D2Q9": ((80, 80, 1), (16, 16, 1)), "D3Q19": ((40, 40, 20), (8, 8, 4)),
                   "D3Q27": ((20, 40, 40), (4, 8, 8))}[lat]
    grid = make_grid(lat, shape, tile)
    m = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    cfg = LBM_Config(m, collision_op=coll, LES=coll == "KBC", DDF_shift=f16, use_float16c=f16, arithmetic="fast")
    flags, bc = ldc_flags(grid, cfg, 0.1)
    tau = 0.55 if coll == "KBC" else 0.8
    f0 = initial_f(grid, cfg, np.random.default_rng(11), tau=tau)
    mask = np.ones(f0.size, bool)
    for k, got, ref, _, _ in step_pairs(grid, cfg, flags, bc, f0, tau, 3):
        check_pop(got, ref, mask, f"clean warps {lat}/{meth}/f16={f16}/{coll} step {k}")


@pytest.mark.parametrize("f16", [False, True])
def test_fast_run_tracks_exact_run(f16):
    """100 free-running steps of the D3Q19 cavity: the fast and the exact builds stay within
    float32 noise of each other (no drift), and the fast run conserves mass as the exact one does."""
    grid = make_grid("D3Q19", (32, 32, 32), (8, 8, 4))
    runs = {}
    for ar in ("exact", "fast"):
        cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, DDF_shift=f16, use_float16c=f16, arithmetic=ar)
        flags, bc = ldc_flags(grid, cfg, 0.1)
        f0 = initial_f(grid, cfg, None)
        s = Solver(grid, cfg)
        fa, fb = to_dev(f0), to_dev(f0)
        bct, flt = to_dev(bc), to_dev(flags)
        s.run(fa, fb, bct, flt, 3 * 0.1 * 31 / 100 + 0.5, 100)
        torch.cuda.synchronize()
        mass = s.mass_momentum(fa, flt)[0]
        runs[ar] = (to_host(fa, f0), mass)
        s.close()
    (fe, me), (ff, mf) = runs["exact"], runs["fast"]
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER)
    flags, _ = ldc_flags(grid, cfg, 0.1)
    mask = fluid_mask_pop(grid, flags)
    if f16:
        de, df = oracle.f16c_decode(fe[mask]).astype(np.float64), oracle.f16c_decode(ff[mask]).astype(np.float64)
        assert np.abs(de - df).max() <= 2e-3 * max(1.0, np.abs(de).max())
    else:
        assert np.abs(fe[mask].astype(np.float64) - ff[mask]).max() <= 2e-5
    assert abs(mf - me) <= 1e-5 * abs(me)
