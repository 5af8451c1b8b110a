"""The reference's CPU-runnable configuration on the GPU library: D2Q9 SRT lid-driven cavity
256 x 256, Re = 100, lid u = 0.1, tau from Re with L = N - 1 (units.mojo:123-126), rest
equilibrium start, pull streaming, 20,000 steps (a CUDA-graph replay), centre lines against the
Re = 100 columns of the Ghia et al. tables the reference ships (tests/golden/ghia_re100.json).
The finer grid than the CPU test's 96^2 tightens the agreement: 0.02 U."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from mojo_lbm_gb300 import LBM_Config, LBM_method
from tests.lbm_cases import ldc_flags, make_grid

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def test_ldc_256_re100_20k_steps_against_ghia():
    import torch

    from mojo_lbm_gb300.solver import Solver
    N, U = 256, 0.1
    g = make_grid("D2Q9", (N, N, 1), (16, 16, 1))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER)
    flags, bc = ldc_flags(g, cfg, U)
    tau = 3 * U * (N - 1) / 100 + 0.5
    s = Solver(g, cfg)
    f = torch.empty(g.num_points * 9, device="cuda")
    s.init_equilibrium(f)
    f2 = f.clone()
    bct, flt = torch.from_numpy(bc).cuda(), torch.from_numpy(flags).cuda()
    s.run(f, f2, bct, flt, tau, 20000, 0)
    rho = torch.empty(g.shape, device="cuda")
    u = torch.empty((2,) + g.shape, device="cuda")
    s.compute_rho_u(rho, u, f, bct, flt)
    u = u.cpu().numpy()
    assert np.isfinite(u).all()
    fix = json.loads((GOLDEN / "ghia_re100.json").read_text())
    coord = lambda t: 0.5 + np.asarray(t) * (N - 2)  # noqa: E731  walls half-way to the solid nodes
    xc = coord(0.5)
    i0 = int(np.floor(xc))
    wx = xc - i0
    ucl = (1 - wx) * u[0, i0, :, 0] + wx * u[0, i0 + 1, :, 0]
    vcl = (1 - wx) * u[1, :, i0, 0] + wx * u[1, :, i0 + 1, 0]
    ys, us = np.array(fix["u_vs_y"]).T
    xs, vs = np.array(fix["v_vs_x"]).T
    inner = (ys > 0) & (ys < 1)
    u_sim = np.interp(coord(ys[inner]), np.arange(N), ucl) / U
    v_sim = np.interp(coord(xs[inner]), np.arange(N), vcl) / U
    assert np.abs(u_sim - us[inner]).max() < 0.02, np.c_[ys[inner], u_sim, us[inner]]
    assert np.abs(v_sim - vs[inner]).max() < 0.02, np.c_[xs[inner], v_sim, vs[inner]]
