"""Error of the float32 step against the float64 oracle for the batched-channel, Taylor-Green LES
and Float16C cavity configurations, on reduced replicas, on the CPU.

The library's float32 kernels equal the float32 oracle bit for bit, Float16C codes included (the
GPU parity tests: every collision operator, LES, the equilibrium outlet, the moving wall and the
link-wise Bouzidi bounce-back), so the float32 oracle's difference from the float64 oracle is the
GPU's.  Reported per step: max |du| over fluid cells relative to the velocity scale, the relative
L2 difference of the (DDF-unshifted) populations of fluid cells, the relative difference of the
float64 sums of rho over fluid cells (float32 vs float64), and the float32 run's own mass change.
Replicas:
  - one channel of the batched workload (224 x 96, Re = 100, parabolic moving-wall inlet with
    u_max = 0.05, equilibrium outlet, a cylinder with Bouzidi links): the mass change is physical
    (the inlet fills the channel against the fixed outlet density);
  - the decaying Taylor-Green vortex with Smagorinsky LES, 32^3 periodic, Re = 1600, u0 = 0.05
    (tau = 0.50048): a closed box, its mass change is the float32 drift;
  - the D3Q19 lid-driven cavity with Float16C storage and DDF shift, 32^3, Re = 100, lid 0.1: the
    velocity error is set by the 11-bit mantissa of the stored codes.
"""
from __future__ import annotations

import math

import numpy as np
import pytest
import torch

import oracle
from mojo_lbm_gb300 import Bounceback_method, LBM_Config, LBM_method, tgv
from mojo_lbm_gb300.workloads import Channel
from tests.lbm_cases import ldc_flags, make_grid

STEPS = 200
REPORT = (1, 25, 50, 100, 150, 200)


def _fluid(grid, flags):
    X, Y, Z = np.meshgrid(*[np.arange(n) for n in grid.shape], indexing="ij")
    return (flags[grid.layouts.flag_offset(X, Y, Z)] & 0x0F) == 0


def _pair(cfg, grid, flags, bc, tau, f32, f64, u_scale, links=None, cfg64=None):
    """Steps the float32 (or Float16C) and float64 oracles side by side; cfg64 is the float64 run's
    configuration (float64 storage with the same DDF shift)."""
    cfg64 = cfg64 or cfg
    bc32, bc64 = bc.astype(np.float32), bc.astype(np.float64)
    a32, b32, a64, b64 = f32, f32.copy(), f64, f64.copy()
    fluid = _fluid(grid, flags)
    f16 = bool(cfg.use_float16c)
    _, w, _ = oracle.lattice(grid.lattice.id)
    w_shift = w[:, None] if cfg.DDF_shift else 0.0  # DDF-shifted storage holds f - w

    def dec(f):
        return (oracle.f16c_decode(f) if f16 else f).astype(np.float64)

    def mass(f):
        rho, _ = oracle.rho_u(cfg64, grid, 64, dec(f), bc64, flags)
        return float(rho[fluid].sum())

    m0 = mass(a32)
    rows = []
    for k in range(STEPS):
        s32, d32 = (a32, b32) if k % 2 == 0 else (b32, a32)
        s64, d64 = (a64, b64) if k % 2 == 0 else (b64, a64)
        oracle.step(cfg, grid, 32, d32, s32, bc32, flags, tau)
        oracle.step(cfg64, grid, 64, d64, s64, bc64, flags, tau)
        if links is not None:
            ids, dirs, dists = links
            for c, prec, f, dt in ((cfg, 32, d32, np.float32), (cfg64, 64, d64, np.float64)):
                oracle.links(c, grid, prec, f, None, ids, dirs, dists.astype(dt), int(Bounceback_method.BOUZIDI),
                             False, 0.0)
        if k + 1 in REPORT:
            g = dec(d32)
            _, u32 = oracle.rho_u(cfg64, grid, 64, g, bc64, flags)
            _, u64 = oracle.rho_u(cfg64, grid, 64, d64, bc64, flags)
            du = max(float(np.abs(u32[d] - u64[d])[fluid].max()) for d in range(grid.D)) / u_scale
            a = oracle.gather(cfg64, grid, 64, g)[:, fluid]
            b = oracle.gather(cfg64, grid, 64, d64)[:, fluid]
            l2 = float(np.linalg.norm(a - b) / np.linalg.norm(b + w_shift))
            rows.append((k + 1, du, l2, mass(d32) / mass(d64) - 1.0, mass(d32) / m0 - 1.0))
    return rows


def _print(name, rows):
    print(f"\n{name}: {STEPS} steps, float32 against the float64 oracle")
    print("  step   max|du|/U     rel L2(f)     mass 32 vs 64   mass change (float32)")
    for r in rows:
        print("  %4d   %.3e    %.3e    %+.3e      %+.3e" % r)


def _channel():
    ch = Channel(224, 96, 100.0, 0.05, 0.02, (16, 16, 1))
    f32 = np.zeros(ch.grid.num_points * 9, np.float32)
    f64 = np.zeros(ch.grid.num_points * 9, np.float64)
    oracle.init(ch.cfg, ch.grid, 32, f32)
    oracle.init(ch.cfg, ch.grid, 64, f64)
    b = ch.body
    links = (b.fluid_boundaries_list.astype(np.int32), b.lattice_links_list.astype(np.int32),
             b.link_distances_list.astype(np.float64))
    assert len(links[0]) > 0
    return _pair(ch.cfg, ch.grid, ch.flags, ch.bc, ch.tau, f32, f64, 0.05, links)


def _tgv():
    N, u0 = 32, 0.05
    grid = make_grid("D3Q19", (N, N, N), (8, 8, 4))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, collision_op="SRT", LES=True)
    tau = 3.0 * u0 * (N / (2.0 * math.pi)) / 1600.0 + 0.5
    u, g = tgv.tgv_fields(N, u0, seed=0, device="cpu", dtype=torch.float64)
    u, g = u.numpy(), g.numpy()
    f32 = np.zeros(grid.num_points * 19, np.float32)
    f64 = np.zeros(grid.num_points * 19, np.float64)
    oracle.init(cfg, grid, 32, f32, 1.0, tau, u, g)
    oracle.init(cfg, grid, 64, f64, 1.0, tau, u, g)
    flags = np.zeros(grid.num_points, np.uint8)
    return _pair(cfg, grid, flags, np.zeros(grid.num_points * 4), tau, f32, f64, u0)


def _ldc_f16c():
    N, U = 32, 0.1
    grid = make_grid("D3Q19", (N, N, N), (8, 8, 4))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, collision_op="SRT", DDF_shift=True, use_float16c=True)
    cfg64 = LBM_Config(LBM_method.DOUBLE_BUFFER, collision_op="SRT", DDF_shift=True)
    flags, bc = ldc_flags(grid, cfg, U)
    tau = 3.0 * U * (N - 1) / 100.0 + 0.5
    f16 = np.zeros(grid.num_points * 19, np.uint16)
    f64 = np.zeros(grid.num_points * 19, np.float64)
    oracle.init(cfg, grid, 32, f16)
    oracle.init(cfg64, grid, 64, f64)
    return _pair(cfg, grid, flags, bc, tau, f16, f64, U, cfg64=cfg64)


# name: case, (max |du|/U, rel L2, mass float32 vs float64) bounds over 200 steps.  float32: the
# differences grow by about 1e-7 (velocity) and 3e-8 (populations, mass) per step; Float16C: the
# codes' rounding (2^-12 of a stored f - w) sets the velocity error from the first steps
CASES = {"channel_d2q9_srt_links_fp32": (_channel, (1e-4, 2e-5, 2e-5)),
         "tgv_d3q19_les_fp32": (_tgv, (1e-4, 2e-5, 2e-5)),
         "ldc_d3q19_f16c": (_ldc_f16c, (5e-4, 2e-5, 2e-5))}


@pytest.mark.parametrize("name", list(CASES))
def test_float32_error_against_float64(name):
    case, (du_bound, l2_bound, m_bound) = CASES[name]
    rows = case()
    _print(name, rows)
    worst_du = max(r[1] for r in rows)
    worst_l2 = max(r[2] for r in rows)
    worst_m = max(abs(r[3]) for r in rows)
    assert worst_du <= du_bound, f"max |du|/U = {worst_du:.3e}"
    assert worst_l2 <= l2_bound, f"rel L2 = {worst_l2:.3e}"
    assert worst_m <= m_bound, f"mass difference = {worst_m:.3e}"
    if name.startswith("tgv"):
        assert abs(rows[-1][4]) <= 2e-5  # closed box: the float32 mass drift
