"""Learned subgrid closure: a per-cell MLP 8 -> 32 -> 32 -> 1 that maps invariants of the
non-equilibrium strain, rho and |u| to an eddy viscosity and replaces Smagorinsky's in the LES
collision.  No counterpart in the reference, whose LES is Smagorinsky with Cs = 0.1
(src/lbm/kernels/ops/turbulence.mojo:12-38).

Training runs on the GPU through the library's own kernels: ``lbm_mlp_forward`` and
``lbm_mlp_backward`` behind a ``torch.autograd.Function`` (torch only computes the loss and its
gradient with respect to the network output), and ``lbm_mlp_adam`` for the update.  Inference
runs inside the collision (``lbm_set_closure``, BF16 tensor-core products); cells whose
normalised features leave the training range keep Smagorinsky.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _capi
from ._capi import check, ptr

N_FEATURES = 8
N_HIDDEN = 32
N_PARAMS = N_FEATURES * N_HIDDEN + N_HIDDEN + N_HIDDEN * N_HIDDEN + N_HIDDEN + N_HIDDEN + 1  # 1377

# Offsets of w1, b1, w2, b2, w3, b3 in the packed parameter vector theta.
_LAYOUT = (("w1", 256), ("b1", 32), ("w2", 1024), ("b2", 32), ("w3", 32), ("b3", 1))


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def init_theta(seed: int = 0, device="cuda") -> torch.Tensor:
    """He-uniform weights, zero biases, a small output layer (so softplus starts near log 2)."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, n in _LAYOUT:
        if name == "w1":
            parts.append(rng.uniform(-1, 1, n) * np.sqrt(6.0 / N_FEATURES))
        elif name == "w2":
            parts.append(rng.uniform(-1, 1, n) * np.sqrt(6.0 / N_HIDDEN))
        elif name == "w3":
            parts.append(rng.uniform(-1, 1, n) * 0.1 / np.sqrt(N_HIDDEN))
        else:
            parts.append(np.zeros(n))
    return torch.tensor(np.concatenate(parts), dtype=torch.float32, device=device)


class MLPFunction(torch.autograd.Function):
    """nu = softplus(MLP_theta(x)) * nu_scale for n rows of 8 normalised features; the gradient
    flows to theta only (the features are data)."""

    @staticmethod
    def forward(ctx, theta: torch.Tensor, x: torch.Tensor, nu_scale: float) -> torch.Tensor:
        if theta.numel() != N_PARAMS or x.dim() != 2 or x.shape[1] != N_FEATURES:
            raise ValueError(f"theta must hold {N_PARAMS} parameters and x be (n, {N_FEATURES})")
        theta = theta.detach().contiguous()
        x = x.detach().contiguous()
        nu = torch.empty(x.shape[0], dtype=torch.float32, device=x.device)
        check(_capi.lib().lbm_mlp_forward(ptr(theta), ptr(x), x.shape[0], float(nu_scale), ptr(nu), _stream()))
        ctx.save_for_backward(theta, x)
        ctx.nu_scale = float(nu_scale)
        return nu

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        theta, x = ctx.saved_tensors
        g = g.detach().contiguous().float()
        grad = torch.empty_like(theta)
        check(_capi.lib().lbm_mlp_backward(ptr(theta), ptr(x), ptr(g), x.shape[0], ctx.nu_scale, ptr(grad),
                                           _stream()))
        return grad, None, None


def mlp(theta: torch.Tensor, x: torch.Tensor, nu_scale: float) -> torch.Tensor:
    return MLPFunction.apply(theta, x, nu_scale)


class Adam:
    """Adam on a flat float32 parameter vector through lbm_mlp_adam."""

    def __init__(self, theta: torch.Tensor, lr: float = 1e-3, betas=(0.9, 0.999), eps: float = 1e-8):
        self.theta = theta
        self.lr, self.beta1, self.beta2, self.eps = float(lr), float(betas[0]), float(betas[1]), float(eps)
        self.m = torch.zeros_like(theta)
        self.v = torch.zeros_like(theta)
        self.t = 0

    def step(self, grad: torch.Tensor) -> None:
        self.t += 1
        check(_capi.lib().lbm_mlp_adam(ptr(self.theta), ptr(grad.contiguous()), ptr(self.m), ptr(self.v),
                                       self.theta.numel(), self.lr, self.beta1, self.beta2, self.eps, self.t,
                                       _stream()))


@dataclass
class Normalisation:
    """x_n = (x - mean) * scale; the training range [lo, hi] of x_n, widened by a margin."""
    mean: np.ndarray
    scale: np.ndarray
    lo: np.ndarray
    hi: np.ndarray

    @staticmethod
    def fit(x: torch.Tensor, margin: float = 0.05) -> "Normalisation":
        x = x.double()
        mean = x.mean(0)
        std = x.std(0)
        # a feature constant over the data (log(tau - 0.5) of a single run) is not scaled
        scale = torch.where(std > 1e-6 * (mean.abs() + 1.0), 1.0 / std, torch.ones_like(std))
        xn = (x - mean) * scale
        lo, hi = xn.min(0).values, xn.max(0).values
        pad = margin * (hi - lo) + 0.01
        return Normalisation(mean.cpu().numpy(), scale.cpu().numpy(), (lo - pad).cpu().numpy(),
                             (hi + pad).cpu().numpy())

    def apply(self, x: torch.Tensor) -> torch.Tensor:
        mean = torch.as_tensor(self.mean, dtype=torch.float32, device=x.device)
        scale = torch.as_tensor(self.scale, dtype=torch.float32, device=x.device)
        return (x.float() - mean) * scale

    def in_range(self, xn: torch.Tensor) -> torch.Tensor:
        lo = torch.as_tensor(self.lo, dtype=torch.float32, device=xn.device)
        hi = torch.as_tensor(self.hi, dtype=torch.float32, device=xn.device)
        return ((xn >= lo) & (xn <= hi)).all(1)


@dataclass
class LearnedClosure:
    """Trained parameters, the output scale and the feature normalisation."""
    theta: torch.Tensor
    nu_scale: float
    norm: Normalisation
    history: list = field(default_factory=list)
    meta: dict = field(default_factory=dict)

    def to_c(self) -> _capi.lbm_closure_t:
        t = self.theta.detach().float().cpu().numpy()
        c = _capi.lbm_closure_t()
        o = 0
        for name, n in _LAYOUT:
            if name == "b3":
                c.b3 = float(t[o])
            else:
                getattr(c, name)[:] = t[o:o + n].tolist()
            o += n
        c.nu_scale = float(self.nu_scale)
        for name, v in (("feat_mean", self.norm.mean), ("feat_scale", self.norm.scale), ("feat_lo", self.norm.lo),
                        ("feat_hi", self.norm.hi)):
            getattr(c, name)[:] = [float(a) for a in v]
        return c

    def predict(self, x_raw: torch.Tensor) -> torch.Tensor:
        """nu_t of raw feature rows through the float32 training kernel (no range check)."""
        with torch.no_grad():
            return mlp(self.theta, self.norm.apply(x_raw).contiguous(), self.nu_scale)

    def save(self, path, meta: dict | None = None) -> None:
        """Parameters and normalisation in an .npz; meta (a JSON-able record of how the network was
        trained and how it scored) rides along."""
        import json
        np.savez(path, theta=self.theta.detach().cpu().numpy(), nu_scale=self.nu_scale, mean=self.norm.mean,
                 scale=self.norm.scale, lo=self.norm.lo, hi=self.norm.hi, meta=json.dumps(meta or {}))

    @staticmethod
    def load(path, device="cuda") -> "LearnedClosure":
        import json
        d = np.load(path)
        c = LearnedClosure(torch.tensor(d["theta"], dtype=torch.float32, device=device), float(d["nu_scale"]),
                           Normalisation(d["mean"], d["scale"], d["lo"], d["hi"]))
        c.meta = json.loads(str(d["meta"])) if "meta" in d.files else {}
        return c


def train(x_raw: torch.Tensor, target: torch.Tensor, *, steps: int = 600, batch: int = 1 << 18, lr: float = 3e-3,
          seed: int = 0, log_every: int = 0) -> LearnedClosure:
    """Fits nu_t(x) to per-cell targets (float32, same device) with Adam on a mean squared error
    scaled by the targets' mean.  Mini-batches are drawn uniformly from the rows."""
    if x_raw.shape[0] != target.shape[0] or x_raw.shape[1] != N_FEATURES:
        raise ValueError("x_raw must be (n, 8) and target (n,)")
    norm = Normalisation.fit(x_raw)
    xn = norm.apply(x_raw).contiguous()
    target = target.float().contiguous()
    nu_scale = float(target.mean().clamp_min(1e-12))
    theta = init_theta(seed, device=x_raw.device)
    opt = Adam(theta, lr=lr)
    gen = torch.Generator(device=x_raw.device)
    gen.manual_seed(seed)
    n = x_raw.shape[0]
    closure = LearnedClosure(theta, nu_scale, norm)
    cosine = lambda k: 0.5 * (1 + np.cos(np.pi * k / steps))  # noqa: E731
    for k in range(steps):
        idx = torch.randint(0, n, (min(batch, n),), device=x_raw.device, generator=gen)
        th = theta.detach().requires_grad_(True)
        nu = mlp(th, xn[idx], nu_scale)
        loss = (((nu - target[idx]) / nu_scale) ** 2).mean()
        loss.backward()
        opt.lr = lr * (0.05 + 0.95 * cosine(k))
        opt.step(th.grad)
        if log_every and (k % log_every == 0 or k == steps - 1):
            closure.history.append((k, float(loss.detach())))
    return closure


def set_closure(solver, closure: LearnedClosure | None) -> None:
    """Installs the closure in an LES Solver (None: back to Smagorinsky)."""
    if closure is None:
        check(solver._lib.lbm_set_closure(solver._h, None))
    else:
        c = closure.to_c()
        check(solver._lib.lbm_set_closure(solver._h, C.byref(c)))
