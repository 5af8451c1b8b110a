"""Error of the GPU step against the float64 oracle, and mass drift, on 64^3 replicas of the
D3Q19 SRT float32 lid-driven cube at Re = 100 and of the D3Q27 KBC + Smagorinsky Float16C
esoteric-pull lid-driven cube at Re = 10000, each in the exact arithmetic (the reference's operation
order) and in the fast arithmetic (LBM_ARITH_FAST), plus the D3Q19 Float16C cube in the fast one.

The GPU runs in its own arithmetic and storage (float32, or Float16C codes with DDF shift); the
oracle runs the same configuration in float64 arithmetic and float64 storage from the same
initial state.  Reported per step: max |u_gpu - u_64| / U_lid over the fluid cells and the
relative L2 difference of the (DDF-unshifted) populations.  Mass drift: the float64 device
reduction of the total mass, relative to its initial value.  The bounds asserted here are the
stated error of each configuration.  Run with -s to print the per-step table."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from mojo_lbm_gb300 import LBM_Config, LBM_method
from mojo_lbm_gb300.solver import Solver
from tests.lbm_cases import ldc_flags, make_grid
from tests.test_gpu_step import to_dev, to_host

pytestmark = pytest.mark.gpu

N = 64
U = 0.1
CASES = {
    # name: lattice, method, collision, LES, Float16C, Re, steps, (max |du|/U bound, rel L2 bound), mass bound,
    #       arithmetic
    # float32: the population error grows ~2e-8 per step with the float32 mass drift (rounding)
    "d3q19_srt_fp32_re100": ("D3Q19", "db", "SRT", False, False, 100.0, 200, (5e-5, 1e-5), 1e-5, "exact"),
    "d3q19_srt_fp32_re100_fast": ("D3Q19", "db", "SRT", False, False, 100.0, 200, (5e-5, 1e-5), 1e-5, "fast"),
    "d3q19_srt_f16c_re100_fast": ("D3Q19", "db", "SRT", False, True, 100.0, 200, (2e-2, 2e-4), 1e-5, "fast"),
    # Float16C at tau = 0.5019: differences of one storage unit grow in the nearly inviscid flow
    "d3q27_kbc_les_f16c_eso_re1e4": ("D3Q27", "eso", "KBC", True, True, 10000.0, 200, (5e-2, 2e-4), 1e-5, "exact"),
    "d3q27_kbc_les_f16c_eso_re1e4_fast": ("D3Q27", "eso", "KBC", True, True, 10000.0, 200, (5e-2, 2e-4), 1e-5,
                                          "fast"),
}


def _fluid_mask(grid, flags):
    """FLUID cells as a [nx, ny, nz] mask (flags are stored in the tiled layout)."""
    X, Y, Z = np.meshgrid(*[np.arange(n) for n in grid.shape], indexing="ij")
    return (flags[grid.layouts.flag_offset(X, Y, Z)] & 0x0F) == 0


def _u_max_err(grid, cfg, f_gpu_dec, f64, bc64, flags, fluid, after_odd):
    """max |u| difference over fluid cells (float64 moments of both lattices)."""
    _, u_g = oracle.rho_u(cfg, grid, 64, f_gpu_dec, bc64, flags, after_odd)
    _, u_r = oracle.rho_u(cfg, grid, 64, f64, bc64, flags, after_odd)
    return float(np.abs(u_g - u_r)[:, fluid].max())


@pytest.mark.parametrize("name", list(CASES))
def test_error_against_float64_oracle_and_mass_drift(name):
    lat, meth, coll, les, f16, Re, steps, (u_bound, l2_bound), mass_bound, arith = CASES[name]
    tile = (8, 8, 4) if lat == "D3Q19" else (4, 8, 8)
    grid = make_grid(lat, (N, N, N), tile)
    method = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    cfg = LBM_Config(method, collision_op=coll, LES=les, DDF_shift=f16, use_float16c=f16, arithmetic=arith)
    cfg64 = LBM_Config(method, collision_op=coll, LES=les, DDF_shift=f16)  # float64 storage, same shift
    flags, bc = ldc_flags(grid, cfg, U)
    tau = 3.0 * U * (N - 1) / Re + 0.5
    # the same initial state: rest equilibrium
    f0 = np.zeros(grid.num_points * grid.Q, oracle.f_dtype(cfg, 32))
    oracle.init(cfg, grid, 32, f0)
    f64 = np.zeros(grid.num_points * grid.Q, np.float64)
    oracle.init(cfg64, grid, 64, f64)
    f64b = f64.copy()
    solver = Solver(grid, cfg)
    assert arith == "exact" or solver.kernel_path in (2, 3)  # the fast arithmetic: block-per-tile kernels
    fa, bct, flt = to_dev(f0), to_dev(bc), to_dev(flags)
    fb = fa.clone()
    bc64 = bc.astype(np.float64)
    m0 = solver.mass_momentum(fa, flt)[0]
    fluid = _fluid_mask(grid, flags)
    _, w, _ = oracle.lattice({"D2Q9": 0, "D3Q19": 1, "D3Q27": 2}[lat])
    w_shift = w[:, None] if f16 else 0.0  # DDF-shifted storage holds f - w
    rows = []
    for k in range(steps):
        if meth == "db":
            src, dst = (fa, fb) if k % 2 == 0 else (fb, fa)
            solver.double_buffer_step(dst, src, bct, flt, tau)
            oracle.step(cfg64, grid, 64, f64b, f64, bc64, flags, tau)
            f64, f64b = f64b, f64
            cur = dst
        else:
            solver.esoteric_pull_step(fa, bct, flt, tau, k % 2 == 0)
            oracle.step(cfg64, grid, 64, f64, f64, bc64, flags, tau, k % 2 == 0)
            cur = fa
        if (k + 1) % 25 == 0 or k == 0:
            g = to_host(cur, f0)
            gd = (oracle.f16c_decode(g) if f16 else g).astype(np.float64)
            after_odd = meth == "eso" and k % 2 == 1  # step k was odd
            a = oracle.gather(cfg64, grid, 64, gd, after_odd)[:, fluid]
            b = oracle.gather(cfg64, grid, 64, f64, after_odd)[:, fluid]
            l2 = float(np.linalg.norm(a - b) / np.linalg.norm(b + w_shift))
            du = _u_max_err(grid, cfg64, gd, f64, bc64, flags, fluid, after_odd)
            mass = solver.mass_momentum(cur if meth == "db" else fa, flt, after_odd)[0]
            rows.append((k + 1, du / U, l2, (mass - m0) / m0))
    torch.cuda.synchronize()
    print(f"\n{name}: {N}^3, tau {tau:.5f}, {steps} steps against the float64 oracle")
    print("  step   max|du|/U     rel L2(f)     mass drift")
    for r in rows:
        print(f"  {r[0]:4d}   {r[1]:.3e}    {r[2]:.3e}    {r[3]:+.3e}")
    worst_u = max(r[1] for r in rows)
    worst_l2 = max(r[2] for r in rows)
    worst_m = max(abs(r[3]) for r in rows)
    assert worst_u <= u_bound, f"max |du|/U = {worst_u:.3e}"
    assert worst_l2 <= l2_bound, f"rel L2 = {worst_l2:.3e}"
    assert worst_m <= mass_bound, f"mass drift = {worst_m:.3e}"
