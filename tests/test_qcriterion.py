"""Q-criterion (calculate_Q_criterion, output/Q_criterion.mojo:90-216).

CPU: the oracle's restatement on a solid-body rotation (vorticity 2 Omega, no strain: Q = Omega^2
in the interior) and on a pure shear built with its non-equilibrium part (Q = 0), and the
reference's edge behaviour (the derivative across a non-periodic domain edge is 0).
GPU: lbm_q_criterion against the oracle, bit for bit, on every lattice, both streaming methods and
both storages, with walls, a moving lid and SOLID cells."""
from __future__ import annotations

import itertools
import zlib

import numpy as np
import pytest

import oracle
from mojo_lbm_gb300 import Flags, LBM_Config, LBM_method
from tests.lbm_cases import initial_f, ldc_flags, make_grid, mixed_flags


def _rotation_state(grid, cfg, omega, tau):
    x = np.arange(grid.nx) - (grid.nx - 1) / 2
    y = np.arange(grid.ny) - (grid.ny - 1) / 2
    X, Y = np.meshgrid(x, y, indexing="ij")
    u = np.zeros((2, grid.nx, grid.ny, 1))
    u[0, ..., 0], u[1, ..., 0] = -omega * Y, omega * X
    f = np.zeros(grid.num_points * grid.Q)
    oracle.init(cfg, grid, 64, f, 1.0, tau, u)
    return f, u


def test_oracle_q_of_solid_body_rotation():
    grid = make_grid("D2Q9", (32, 32, 1), (16, 16, 1))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, include_moving_boundary=False)
    omega, tau = 1e-3, 1.0
    f, u_init = _rotation_state(grid, cfg, omega, tau)
    flags = np.zeros(grid.num_points, np.uint8)
    bc = np.zeros(grid.num_points * 3)
    rho, u = oracle.rho_u(cfg, grid, 64, f, bc, flags)
    q = oracle.q_criterion(cfg, grid, 64, f, bc, flags, u, tau)
    inner = q[3:-3, 3:-3, 0]
    assert np.allclose(inner, omega ** 2, rtol=1e-4)


def test_oracle_q_edge_derivative_is_zero():
    """Populations at rest (no strain) with the rotation given as the velocity field: Q is the
    vorticity term alone.  Across a non-periodic domain edge the reference's weighting drops the
    derivative, so on the x = 0 column omega = -du/dy only: Q = Omega^2 / 4."""
    grid = make_grid("D2Q9", (32, 32, 1), (16, 16, 1))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, include_moving_boundary=False)
    omega = 1e-3
    f = np.zeros(grid.num_points * grid.Q)
    oracle.init(cfg, grid, 64, f)
    _, u = _rotation_state(grid, cfg, omega, 1.0)
    flags = np.zeros(grid.num_points, np.uint8)
    bc = np.zeros(grid.num_points * 3)
    q = oracle.q_criterion(cfg, grid, 64, f, bc, flags, u, 1.0)
    assert np.allclose(q[1:-1, 1:-1, 0], omega ** 2, rtol=1e-12)
    assert np.allclose(q[0, 1:-1, 0], 0.25 * omega ** 2, rtol=1e-12)
    assert np.allclose(q[1:-1, -1, 0], 0.25 * omega ** 2, rtol=1e-12)
    assert np.allclose(q[0, 0, 0], 0.0, atol=1e-20)  # both derivatives dropped at a corner


def test_oracle_q_of_pure_shear_is_zero():
    grid = make_grid("D2Q9", (32, 32, 1), (16, 16, 1))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, include_moving_boundary=False)
    gamma, tau = 1e-3, 1.0
    y = np.arange(grid.ny) - (grid.ny - 1) / 2
    u = np.zeros((2,) + grid.shape)
    u[0] = gamma * y[None, :, None]
    grad = np.zeros((4,) + grid.shape)
    grad[1] = gamma  # du_x / dy
    f = np.zeros(grid.num_points * grid.Q)
    oracle.init(cfg, grid, 64, f, 1.0, tau, u, grad)
    flags = np.zeros(grid.num_points, np.uint8)
    bc = np.zeros(grid.num_points * 3)
    _, uo = oracle.rho_u(cfg, grid, 64, f, bc, flags)
    q = oracle.q_criterion(cfg, grid, 64, f, bc, flags, uo, tau)
    # |omega|^2 / 4 = gamma^2 / 4 against |S|^2 / 2 = gamma^2 / 4 (S from the streamed populations)
    assert np.abs(q[3:-3, 3:-3, 0]).max() < 0.15 * gamma ** 2


CASES = list(itertools.product(["D2Q9", "D3Q19", "D3Q27"], ["db", "eso"], ["fp32", "f16c"], ["mixed", "ldc"]))
SHAPES = {"D2Q9": ((30, 20, 1), (10, 5, 1)), "D3Q19": ((18, 12, 10), (6, 4, 5)), "D3Q27": ((12, 12, 10), (4, 6, 5))}


@pytest.mark.gpu
@pytest.mark.parametrize("lat,meth,store,case", CASES, ids=["-".join(c) for c in CASES])
def test_gpu_q_criterion_matches_oracle(lat, meth, store, case):
    import torch

    from mojo_lbm_gb300.solver import Solver
    from tests.test_gpu_step import to_dev
    shape, tile = SHAPES[lat]
    grid = make_grid(lat, shape, tile)
    f16 = store == "f16c"
    method = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    rng = np.random.default_rng(zlib.crc32(f"qcrit/{lat}/{meth}/{store}/{case}".encode()))
    if case == "mixed":
        cfg = LBM_Config(method, BCs={Flags.EQUILIBRIUM}, DDF_shift=f16, use_float16c=f16)
        flags, bc = mixed_flags(grid, rng)
    else:
        cfg = LBM_Config(method, DDF_shift=f16, use_float16c=f16)
        flags, bc = ldc_flags(grid, cfg, 0.1)
    f0 = initial_f(grid, cfg, rng, tau=0.8)
    s = Solver(grid, cfg)
    ft, bct, flt = to_dev(f0), to_dev(bc), to_dev(flags)
    D = grid.D
    for after_odd in ([False] if meth == "db" else [False, True]):
        rho = torch.empty(grid.shape, device="cuda")
        u = torch.empty((D,) + grid.shape, device="cuda")
        q = torch.full(grid.shape, float("nan"), device="cuda")
        s.compute_rho_u(rho, u, ft, bct, flt, after_odd)
        s.q_criterion(q, ft, bct, flt, u, 0.8, after_odd)
        torch.cuda.synchronize()
        _, u_ref = oracle.rho_u(cfg, grid, 32, f0, bc, flags, after_odd)
        q_ref = oracle.q_criterion(cfg, grid, 32, f0, bc, flags, u_ref, 0.8, after_odd)
        got = q.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), q_ref.view(np.uint32)), \
            f"{int(np.sum(got.view(np.uint32) != q_ref.view(np.uint32)))} cells differ"
