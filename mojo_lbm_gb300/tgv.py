"""Decaying Taylor–Green vortex in a periodic box: the flow the learned closure is trained and
evaluated on.

A fine D3Q19 run is box-filtered onto the grid of half its resolution; the filtered fields give
the closure's training pairs (strain invariants -> the eddy viscosity that best explains the
subgrid stress) and the reference against which coarse LES runs (Smagorinsky, learned) are
measured by kinetic energy and energy spectrum.  Conventions: the box is [0, 2 pi)^3 with N cells
per side, L = N / (2 pi) cells, u0 the lattice velocity amplitude, Re = u0 L / nu, one
convective time unit L / u0 steps.  The initial field is the analytic vortex
u = u0 sin x cos y cos z, v = -u0 cos x sin y cos z, w = 0 plus a seeded divergence-free
perturbation of low-wavenumber Fourier modes, evaluated at cell centres (i + 1/2) 2 pi / N so
that a fine run and its coarse counterpart start from the same continuous field; the initial
populations are f_eq + f_neq from the analytic velocity gradient.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np
import torch
import torch.nn.functional as F

from .config import LBM_Config
from .constants import LBM_method
from .grid import LBM_Grid
from .lattice import get_D3Q19
from .solver import Solver

# ---------------------------------------------------------------------------------------------
# initial field
# ---------------------------------------------------------------------------------------------


def _modes(seed: int, n_modes: int = 8, kmax: int = 3):
    """Seeded divergence-free Fourier modes: wavevector k (integers), amplitude a with a.k = 0,
    phase; amplitudes sum to 1 so the perturbation never exceeds the requested amplitude."""
    rng = np.random.default_rng(seed)
    ks, amps, phases = [], [], []
    while len(ks) < n_modes:
        k = rng.integers(-kmax, kmax + 1, 3)
        if not k.any():
            continue
        a = rng.normal(size=3)
        a -= k * (a @ k) / (k @ k)
        ks.append(k.astype(np.float64))
        amps.append(a)
        phases.append(rng.uniform(0, 2 * np.pi))
    amps = np.array(amps)
    amps /= np.abs(amps).sum(1).sum()
    return np.array(ks), amps, np.array(phases)


def tgv_fields(N: int, u0: float, seed: int = 0, amp: float = 1e-3, device="cuda", dtype=torch.float32):
    """Velocity u[3][N][N][N] and gradient g[9][N][N][N] (du_a/dx_b at a*3+b, per cell) of the
    perturbed vortex in lattice units."""
    h = 2 * math.pi / N
    x = (torch.arange(N, device=device, dtype=torch.float64) + 0.5) * h
    X, Y, Z = torch.meshgrid(x, x, x, indexing="ij")
    sx, cx, sy, cy, sz, cz = torch.sin(X), torch.cos(X), torch.sin(Y), torch.cos(Y), torch.sin(Z), torch.cos(Z)
    u = torch.zeros((3, N, N, N), dtype=torch.float64, device=device)
    g = torch.zeros((9, N, N, N), dtype=torch.float64, device=device)
    u[0] = u0 * sx * cy * cz
    u[1] = -u0 * cx * sy * cz
    g[0] = u0 * cx * cy * cz * h
    g[1] = -u0 * sx * sy * cz * h
    g[2] = -u0 * sx * cy * sz * h
    g[3] = u0 * sx * sy * cz * h
    g[4] = -u0 * cx * cy * cz * h
    g[5] = u0 * cx * sy * sz * h
    del sx, cx, sy, cy, sz, cz
    ks, amps, phases = _modes(seed)
    for k, a, ph in zip(ks, amps, phases):
        arg = k[0] * X + k[1] * Y + k[2] * Z + ph
        c, s = torch.cos(arg), torch.sin(arg)
        for i in range(3):
            u[i] += amp * u0 * a[i] * c
            for j in range(3):
                g[i * 3 + j] -= amp * u0 * a[i] * k[j] * s * h
    return u.to(dtype).contiguous(), g.to(dtype).contiguous()


# ---------------------------------------------------------------------------------------------
# filtering, strain, spectra
# ---------------------------------------------------------------------------------------------


def box2(a: torch.Tensor) -> torch.Tensor:
    """Mean over 2x2x2 blocks of the last three axes (the box filter of width two fine cells,
    sampled on the coarse grid)."""
    s = a.shape
    n = s[-1] // 2
    return a.reshape(*s[:-3], n, 2, n, 2, n, 2).mean(dim=(-5, -3, -1))


def _ddx(a: torch.Tensor, axis: int) -> torch.Tensor:
    """Fourth-order central difference along axis (periodic, unit spacing)."""
    return (8 * (torch.roll(a, -1, axis) - torch.roll(a, 1, axis))
            - (torch.roll(a, -2, axis) - torch.roll(a, 2, axis))) / 12.0


def strain(u: torch.Tensor) -> torch.Tensor:
    """S[6][...] in stress order xx, xy, xz, yy, yz, zz from u[3][n][n][n] (periodic)."""
    ax = (-3, -2, -1)
    d = [[_ddx(u[i], ax[j]) for j in range(3)] for i in range(3)]
    return torch.stack([d[0][0], 0.5 * (d[0][1] + d[1][0]), 0.5 * (d[0][2] + d[2][0]), d[1][1],
                        0.5 * (d[1][2] + d[2][1]), d[2][2]])


_PAIRS = ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))


def features(S: torch.Tensor, rho: torch.Tensor, u: torch.Tensor, tau: float) -> torch.Tensor:
    """The closure's eight features per cell (rows), from S[6], rho and u[3] on one grid; the
    same definitions as the collision kernel's (include/lbm_gb300.h, lbm_closure_t)."""
    S = S.double()
    s2 = sum((S[n] ** 2) * (1.0 if a == b else 2.0) for n, (a, b) in enumerate(_PAIRS))
    q = 2 * s2 + 1e-24
    sq = torch.sqrt(q)
    tr = S[0] + S[3] + S[5]
    m = tr / 3
    a, b, c = S[0] - m, S[3] - m, S[5] - m
    det = a * (b * c - S[4] ** 2) - S[1] * (S[1] * c - S[4] * S[2]) + S[2] * (S[1] * S[4] - b * S[2])
    off = 2 * (S[1] ** 2 + S[2] ** 2 + S[4] ** 2)
    uu = (u.double() ** 2).sum(0)
    x = torch.stack([torch.log(q) / 2, tr / sq, det / (q * sq), rho.double() - 1, torch.sqrt(uu), 2 * off / q,
                     torch.full_like(uu, math.log(tau - 0.5)), uu / sq])
    return x.reshape(8, -1).T.float().contiguous()


def _box3(a: torch.Tensor) -> torch.Tensor:
    """Periodic 3x3x3 mean."""
    p = F.pad(a[None, None], (1, 1, 1, 1, 1, 1), mode="circular")
    return F.avg_pool3d(p, 3, stride=1)[0, 0]


def sgs_target(u_fine: torch.Tensor, u_bar: torch.Tensor, S_bar: torch.Tensor) -> torch.Tensor:
    """Eddy viscosity that best explains the subgrid stress tau_ab = bar(u_a u_b) - bar(u_a)
    bar(u_b) in the least-squares sense, nu_t = max(0, -<tau^d : S> / <2 S : S>), with <.> a
    periodic 3x3x3 mean (coarse lattice units)."""
    num = torch.zeros_like(u_bar[0], dtype=torch.float64)
    tr = torch.zeros_like(num)
    taus = []
    for (a, b) in _PAIRS:
        t = (box2(u_fine[a] * u_fine[b]) - u_bar[a] * u_bar[b]).double()
        taus.append(t)
        if a == b:
            tr += t
    for n, (a, b) in enumerate(_PAIRS):
        t = taus[n] - (tr / 3 if a == b else 0)
        num -= t * S_bar[n].double() * (1.0 if a == b else 2.0)
    den = 2 * sum((S_bar[n].double() ** 2) * (1.0 if a == b else 2.0) for n, (a, b) in enumerate(_PAIRS))
    return torch.clamp(_box3(num) / (_box3(den) + 1e-30), min=0.0).float()


def energy_spectrum(u: torch.Tensor) -> torch.Tensor:
    """E(k) for integer shells k = 0 .. N/2 of u[3][N][N][N] (float64; sum_k E(k) = mean 0.5|u|^2
    up to the shells beyond N/2)."""
    N = u.shape[-1]
    uh = torch.fft.fftn(u.double(), dim=(-3, -2, -1)) / N ** 3
    e = 0.5 * (uh.real ** 2 + uh.imag ** 2).sum(0)
    k = torch.fft.fftfreq(N, 1.0 / N, device=u.device)
    K = torch.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2)
    shell = torch.round(K).long().clamp(max=N // 2 + 1)
    E = torch.zeros(N // 2 + 2, dtype=torch.float64, device=u.device)
    E.index_add_(0, shell.ravel(), e.ravel())
    return E[: N // 2 + 1]


def kinetic_energy(u: torch.Tensor) -> float:
    return float(0.5 * (u.double() ** 2).sum(0).mean())


# ---------------------------------------------------------------------------------------------
# runs
# ---------------------------------------------------------------------------------------------


@dataclass
class TGVCase:
    N: int
    Re: float = 1600.0
    u0: float = 0.05

    @property
    def L(self) -> float:
        return self.N / (2 * math.pi)

    @property
    def tau(self) -> float:
        return 3.0 * self.u0 * self.L / self.Re + 0.5

    def steps(self, t_star: float) -> int:
        return int(round(float(t_star) * self.L / self.u0))


class TGVRun:
    """One periodic D3Q19 run (double buffer, pull) with rho/u read-back at requested times."""

    def __init__(self, case: TGVCase, *, seed: int = 0, amp: float = 1e-3, les: str | None = None, Cs: float = 0.1,
                 closure=None, collision: str = "SRT", tile=(8, 8, 4), device="cuda"):
        self.case = case
        N = case.N
        self.grid = LBM_Grid(get_D3Q19(), N, N, N, tile)
        self.cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, collision_op=collision, LES=les is not None, Cs=Cs,
                              include_moving_boundary=False)
        self.solver = Solver(self.grid, self.cfg)
        if les == "learned":
            from .closure import set_closure
            set_closure(self.solver, closure)
        elif les not in (None, "smagorinsky"):
            raise ValueError("les must be None, 'smagorinsky' or 'learned'")
        n = self.grid.num_points
        self.f = [torch.empty(n * 19, dtype=torch.float32, device=device) for _ in range(2)]
        self.bc = torch.zeros(n * 4, dtype=torch.float32, device=device)
        self.flags = torch.zeros(n, dtype=torch.uint8, device=device)
        u, g = tgv_fields(N, case.u0, seed, amp, device)
        self.solver.init_equilibrium(self.f[0], 1.0, case.tau, u, g)
        del u, g
        self.step = 0
        self.rho = torch.empty((N, N, N), dtype=torch.float32, device=device)
        self.u = torch.empty((3, N, N, N), dtype=torch.float32, device=device)

    def advance_to(self, step: int) -> None:
        if step > self.step:
            self.solver.run(self.f[0], self.f[1], self.bc, self.flags, self.case.tau, step - self.step, self.step)
            self.step = step

    def fields(self):
        self.solver.compute_rho_u(self.rho, self.u, self.f[self.step % 2], self.bc, self.flags)
        return self.rho, self.u

    def time_steps(self, n_steps: int) -> float:
        """Seconds per step over n_steps graph-replayed steps (CUDA events, after one warm-up chunk)."""
        self.advance_to(self.step + 64)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(torch.cuda.default_stream())
        self.solver.run(self.f[0], self.f[1], self.bc, self.flags, self.case.tau, n_steps, self.step)
        e1.record(torch.cuda.default_stream())
        e1.synchronize()
        self.step += n_steps
        return e0.elapsed_time(e1) * 1e-3 / n_steps


def reference_snapshots(fine: TGVCase, t_stars, *, seed: int, amp: float = 1e-3, train: bool = False,
                        samples_per_snapshot: int = 1 << 21, collision: str = "SRT", tile=(8, 8, 4)):
    """Runs the fine case and returns, per t*, the box-filtered fields on the coarse grid (rho, u)
    and, if train, (features, targets) sampled from the coarse cells."""
    coarse = TGVCase(fine.N // 2, fine.Re, fine.u0)
    run = TGVRun(fine, seed=seed, amp=amp, collision=collision, tile=tile)
    out = {}
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    for t in t_stars:
        run.advance_to(2 * coarse.steps(t))  # fine step 2k is coarse step k
        rho_f, u_f = run.fields()
        rho_b, u_b = box2(rho_f), box2(u_f)
        item = {"rho": rho_b.clone(), "u": u_b.clone(), "finite": bool(torch.isfinite(u_f).all())}
        if train:
            S_b = strain(u_b)
            nu = sgs_target(u_f, u_b, S_b).reshape(-1)
            x = features(S_b, rho_b, u_b, coarse.tau)
            idx = torch.randint(0, x.shape[0], (min(samples_per_snapshot, x.shape[0]),), device="cuda",
                                generator=gen)
            item["x"], item["nu"] = x[idx].contiguous(), nu[idx].contiguous()
        out[t] = item
    del run
    torch.cuda.empty_cache()
    return out


def les_snapshots(coarse: TGVCase, t_stars, *, seed: int, les: str, closure=None, Cs: float = 0.1,
                  amp: float = 1e-3, collision: str = "SRT", tile=(8, 8, 4)):
    """Coarse LES (Smagorinsky or learned) fields at each t*."""
    run = TGVRun(coarse, seed=seed, amp=amp, les=les, closure=closure, Cs=Cs, collision=collision, tile=tile)
    out = {}
    for t in t_stars:
        run.advance_to(coarse.steps(t))
        rho, u = run.fields()
        out[t] = {"rho": rho.clone(), "u": u.clone(), "finite": bool(torch.isfinite(u).all())}
    return out


def spectrum_error(les: dict, ref: dict, t_stars, k_min: int = 1, k_max: int | None = None) -> float:
    """Mean over the times and the shells k_min..k_max of |log E_les(k) - log E_ref(k)|."""
    errs = []
    for t in t_stars:
        if not les[t]["finite"]:
            return float("inf")
        E, R = energy_spectrum(les[t]["u"]), energy_spectrum(ref[t]["u"])
        hi = k_max or (E.numel() - 2)
        errs.append(torch.abs(torch.log(E[k_min:hi + 1]) - torch.log(R[k_min:hi + 1])).mean().item())
    return float(np.mean(errs))


def energy_error(les: dict, ref: dict, t_stars) -> float:
    """Mean over the times of |KE_les - KE_ref| / KE_ref."""
    errs = []
    for t in t_stars:
        if not les[t]["finite"]:
            return float("inf")
        errs.append(abs(kinetic_energy(les[t]["u"]) - kinetic_energy(ref[t]["u"])) / kinetic_energy(ref[t]["u"]))
    return float(np.mean(errs))


def study(N_fine: int = 512, Re: float = 1600.0, u0: float = 0.05, *, train_times=(2, 4, 6, 8, 10),
          eval_times=(2, 4, 6, 8, 10), train_seed: int = 1, eval_seed: int = 0, train_steps: int = 600,
          time_steps: int = 256, collision: str = "SRT", log=print) -> dict:
    """The whole comparison: fine reference runs (training seed, evaluation seed), training,
    coarse Smagorinsky and learned runs, their errors and their per-step times."""
    fine = TGVCase(N_fine, Re, u0)
    coarse = TGVCase(N_fine // 2, Re, u0)
    t0 = time.time()
    tr = reference_snapshots(fine, train_times, seed=train_seed, train=True, collision=collision)
    x = torch.cat([tr[t]["x"] for t in train_times])
    nu = torch.cat([tr[t]["nu"] for t in train_times])
    del tr
    log(f"training data: {x.shape[0]} samples, mean nu_t {float(nu.mean()):.3e} ({time.time() - t0:.0f} s)")
    from .closure import train
    closure = train(x, nu, steps=train_steps, log_every=100)
    del x, nu
    log(f"trained: loss {closure.history[0][1]:.4f} -> {closure.history[-1][1]:.4f} ({time.time() - t0:.0f} s)")
    ref = reference_snapshots(fine, eval_times, seed=eval_seed, collision=collision)
    smag = les_snapshots(coarse, eval_times, seed=eval_seed, les="smagorinsky", collision=collision)
    learned = les_snapshots(coarse, eval_times, seed=eval_seed, les="learned", closure=closure, collision=collision)
    res = {
        "N_fine": N_fine, "N_coarse": coarse.N, "Re": Re, "u0": u0, "tau_coarse": coarse.tau, "tau_fine": fine.tau,
        "eval_times": list(eval_times),
        "spectrum_error": {"smagorinsky": spectrum_error(smag, ref, eval_times),
                           "learned": spectrum_error(learned, ref, eval_times)},
        "energy_error": {"smagorinsky": energy_error(smag, ref, eval_times),
                         "learned": energy_error(learned, ref, eval_times)},
        "ke": {"reference": [kinetic_energy(ref[t]["u"]) for t in eval_times],
               "smagorinsky": [kinetic_energy(smag[t]["u"]) for t in eval_times],
               "learned": [kinetic_energy(learned[t]["u"]) for t in eval_times]},
    }
    del ref, smag, learned
    torch.cuda.empty_cache()
    if time_steps:
        s = TGVRun(coarse, seed=eval_seed, les="smagorinsky", collision=collision).time_steps(time_steps)
        l_run = TGVRun(coarse, seed=eval_seed, les="learned", closure=closure, collision=collision)
        lt = l_run.time_steps(time_steps)
        res["s_per_step"] = {"smagorinsky": s, "learned": lt}
        res["mlups"] = {"smagorinsky": coarse.N ** 3 / s / 1e6, "learned": coarse.N ** 3 / lt / 1e6}
        res["time_ratio"] = lt / s
    res["closure"] = closure
    return res


def main(argv=None) -> None:
    """Runs the comparison and prints one JSON line (and saves the trained closure with --save)."""
    import argparse
    import json
    ap = argparse.ArgumentParser(description="Learned closure vs Smagorinsky on the decaying Taylor-Green vortex")
    ap.add_argument("--fine", type=int, default=512, help="cells per side of the fine reference run")
    ap.add_argument("--re", type=float, default=1600.0)
    ap.add_argument("--u0", type=float, default=0.05)
    ap.add_argument("--train-times", default="2,4,6,8,10")
    ap.add_argument("--eval-times", default="2,4,6,8,10")
    ap.add_argument("--train-steps", type=int, default=600)
    ap.add_argument("--time-steps", type=int, default=400)
    ap.add_argument("--collision", default="SRT")
    ap.add_argument("--save", default="", help="path of an .npz for the trained closure")
    args = ap.parse_args(argv)
    times = lambda s: tuple(float(t) for t in s.split(","))  # noqa: E731
    res = study(args.fine, args.re, args.u0, train_times=times(args.train_times), eval_times=times(args.eval_times),
                train_steps=args.train_steps, time_steps=args.time_steps, collision=args.collision,
                log=lambda *a: print(*a, flush=True))
    closure = res.pop("closure")
    res["train_loss"] = closure.history
    res["command"] = "python -m mojo_lbm_gb300.tgv " + " ".join(argv if argv is not None else __import__("sys").argv[1:])
    if args.save:
        closure.save(args.save, meta=res)
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
