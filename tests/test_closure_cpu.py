"""Host-side checks of the learned closure: the float64 numpy network (the oracle of the CUDA
training kernels) against central finite differences, the C++ oracle's closure (BF16 emulation)
against the numpy network, the feature definitions of the oracle against the package's training
features, the packing of lbm_closure_t, and the Smagorinsky fallback of the oracle's LES step."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from oracle import closure as ref
from mojo_lbm_gb300 import LBM_Config, LBM_method
from mojo_lbm_gb300 import tgv
from mojo_lbm_gb300.closure import N_PARAMS, LearnedClosure, Normalisation, init_theta
from tests.lbm_cases import initial_f, ldc_flags, make_grid


def _theta(seed=0):
    return init_theta(seed, device="cpu").double().numpy() + np.random.default_rng(seed).normal(0, 0.05, N_PARAMS)


def test_numpy_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    theta = _theta(1)
    x = rng.normal(size=(64, 8))
    g = rng.normal(size=64)
    nu_scale = 2e-3
    grad = ref.backward(theta, x, g, nu_scale)
    h = 1e-6
    for p in rng.choice(N_PARAMS, 60, replace=False).tolist() + [N_PARAMS - 1, 0, 300]:
        tp, tm = theta.copy(), theta.copy()
        tp[p] += h
        tm[p] -= h
        fd = (g @ ref.forward(tp, x, nu_scale)[0] - g @ ref.forward(tm, x, nu_scale)[0]) / (2 * h)
        assert abs(fd - grad[p]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (p, fd, grad[p])


def test_numpy_adam_first_step_is_sign_times_lr():
    g = np.array([1e-3, -2.0, 0.5])
    th, m, v = ref.adam(np.zeros(3), g, np.zeros(3), np.zeros(3), 0.1, 0.9, 0.999, 1e-12, 1)
    assert np.allclose(th, -0.1 * np.sign(g))


def _closure_struct(theta, nu_scale=1e-3, lo=-1e30, hi=1e30):
    return oracle.closure_struct(theta, nu_scale, np.zeros(8), np.ones(8), np.full(8, lo), np.full(8, hi))


def test_oracle_closure_matches_numpy_network_within_bf16():
    """The oracle rounds weights and activations to BF16 like the tensor cores; the float64
    network agrees to BF16 precision."""
    rng = np.random.default_rng(2)
    theta = _theta(2)
    n = 200
    S = rng.normal(0, 1e-3, (n, 6))
    s2 = (S[:, [0, 3, 5]] ** 2).sum(1) + 2 * (S[:, [1, 2, 4]] ** 2).sum(1)
    rho = rng.uniform(0.98, 1.02, n)
    uu = rng.uniform(0, 0.01, n)
    tau = np.full(n, 0.51)
    oracle.set_closure(_closure_struct(theta))
    try:
        x, nu = oracle.closure_eval(3, 64, S, s2, rho, uu, tau)
    finally:
        oracle.set_closure(None)
    want = ref.forward(theta, x, 1e-3)[0]
    assert np.all(nu >= 0)
    assert np.allclose(nu, want, rtol=3e-2, atol=1e-6)


@pytest.mark.parametrize("D", [2, 3])
def test_oracle_features_match_training_features(D):
    """The features the collision computes (oracle restatement) and the ones the training data
    uses (mojo_lbm_gb300.tgv.features) are the same functions of (S, rho, u, tau)."""
    rng = np.random.default_rng(3 + D)
    n = 500
    ns = 6 if D == 3 else 3
    S = rng.normal(0, 1e-3, (n, ns))
    u = rng.normal(0, 0.03, (3, n))
    if D == 2:
        u[2] = 0
    rho = rng.uniform(0.98, 1.02, n)
    tau = 0.5123
    if D == 2:  # embed the 2D tensor (xx, xy, yy) in 3D stress order with zero z components
        S3 = np.zeros((n, 6))
        S3[:, 0], S3[:, 1], S3[:, 3] = S[:, 0], S[:, 1], S[:, 2]
        pairs = [(0, 1.0), (1, 2.0), (2, 1.0)]
    else:
        S3 = S
        pairs = [(0, 1.0), (1, 2.0), (2, 2.0), (3, 1.0), (4, 2.0), (5, 1.0)]
    s2 = sum(w * S[:, k] ** 2 for k, w in pairs)
    uu = (u ** 2).sum(0)
    x_or, _ = oracle.closure_eval(D, 64, S, s2, rho, uu, np.full(n, tau))
    x_py = tgv.features(torch.from_numpy(S3.T.copy()), torch.from_numpy(rho), torch.from_numpy(u), tau).double().numpy()
    if D == 2:
        # the 2D deviator uses the 2D mean (tr/2): det and the trace-based features differ by
        # definition from the 3D embedding; compare the dimension-independent ones
        cols = [0, 1, 3, 4, 5, 6, 7]
    else:
        cols = list(range(8))
    assert np.allclose(x_or[:, cols], x_py[:, cols], rtol=2e-6, atol=1e-6)


def test_closure_packing_matches_oracle_struct():
    theta = torch.from_numpy(_theta(4).astype(np.float32))
    norm = Normalisation(np.arange(8.0), np.ones(8) * 2, -np.ones(8) * 3, np.ones(8) * 4)
    c = LearnedClosure(theta, 1.5e-3, norm).to_c()
    o = oracle.closure_struct(theta.numpy(), 1.5e-3, norm.mean, norm.scale, norm.lo, norm.hi)
    assert C.sizeof(c) == C.sizeof(o) == 4 * (N_PARAMS + 1 + 32)
    assert bytes(c) == bytes(o)


def test_normalisation_handles_constant_feature():
    x = torch.randn(1000, 8, dtype=torch.float64, generator=torch.Generator().manual_seed(6))
    x[:, 6] = -5.57
    n = Normalisation.fit(x)
    xn = n.apply(x)
    assert torch.isfinite(xn).all()
    assert bool(n.in_range(xn).all())
    assert n.scale[6] == 1.0 and n.lo[6] < 0 < n.hi[6]


def test_oracle_les_step_out_of_range_closure_is_smagorinsky():
    """A closure whose training range excludes every cell leaves the LES step unchanged."""
    grid = make_grid("D3Q19", (16, 8, 8), (8, 4, 4))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, LES=True)
    flags, bc = ldc_flags(grid, cfg, 0.1)
    f0 = initial_f(grid, cfg, np.random.default_rng(6), tau=0.52)
    a, b = np.zeros_like(f0), np.zeros_like(f0)
    oracle.step(cfg, grid, 32, a, f0, bc.copy(), flags, 0.52)
    oracle.set_closure(_closure_struct(_theta(6), lo=1.0, hi=-1.0))
    try:
        oracle.step(cfg, grid, 32, b, f0, bc.copy(), flags, 0.52)
    finally:
        oracle.set_closure(None)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_oracle_les_step_with_closure_changes_tau():
    grid = make_grid("D3Q19", (16, 8, 8), (8, 4, 4))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, LES=True)
    flags, bc = ldc_flags(grid, cfg, 0.1)
    f0 = initial_f(grid, cfg, np.random.default_rng(7), tau=0.52)
    a, b = np.zeros_like(f0), np.zeros_like(f0)
    oracle.step(cfg, grid, 32, a, f0, bc.copy(), flags, 0.52)
    oracle.set_closure(_closure_struct(_theta(7), nu_scale=5e-3))
    try:
        oracle.step(cfg, grid, 32, b, f0, bc.copy(), flags, 0.52)
    finally:
        oracle.set_closure(None)
    assert np.isfinite(b).all()
    assert not np.array_equal(a, b)
