"""TEST INFRASTRUCTURE — ctypes wrapper of the CPU oracle (liblbm_oracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module, as
the values the tests compare against or as the timed CPU baseline; the product never does.  Parity with the reference
is UNPINNED (see lbm_oracle.cpp): the reference is Mojo and its repository has no golden
vectors for the step; the oracle is pinned to the Ghia et al. cavity fixture, the DFG drag the
reference recorded, and invariants.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liblbm_oracle.so"

_lib = None


def build(force: bool = False) -> Path:
    """Compiles the oracle with its Makefile (g++, OpenMP)."""
    src = [HERE / "lbm_oracle.cpp", HERE / "Makefile", HERE.parent / "include" / "lbm_gb300.h"]
    if force or not LIB.exists() or any(p.stat().st_mtime > LIB.stat().st_mtime for p in src):
        subprocess.run(["make", "-s", "-C", str(HERE), "-B" if force else "liblbm_oracle.so"], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        h = C.CDLL(str(LIB))
        vp, i32, i64, f64 = C.c_void_p, C.c_int, C.c_int64, C.c_double
        h.oracle_step.argtypes = [vp, vp, i32, vp, vp, vp, vp, f64, i32, i32]
        h.oracle_step_range.argtypes = [vp, vp, i32, vp, vp, vp, vp, f64, i32, i32, i64, i64]
        h.oracle_init.argtypes = [vp, vp, i32, vp, f64, f64, vp, vp]
        h.oracle_rho_u.argtypes = [vp, vp, i32, vp, vp, vp, vp, vp, i32]
        h.oracle_links.argtypes = [vp, vp, i32, vp, vp, vp, vp, vp, i64, i32, i32, f64]
        h.oracle_drag.argtypes = [vp, vp, i32, vp, vp, vp, vp, i64]
        h.oracle_gather.argtypes = [vp, vp, i32, vp, vp, i32]
        h.oracle_f16c_encode.argtypes = [vp, vp, i64]
        h.oracle_f16c_decode.argtypes = [vp, vp, i64]
        h.oracle_layout_offset.argtypes = [vp, i64, i64, i64, i64, i64]
        h.oracle_stress_pairs.argtypes = [i32, vp]
        h.oracle_layout_offset.restype = i64
        h.oracle_lattice.argtypes = [i32, vp, vp, vp]
        h.oracle_max_threads.restype = i32
        h.oracle_set_closure.argtypes = [vp]
        h.oracle_q_criterion.argtypes = [vp, vp, i32, vp, vp, vp, vp, f64, i32, vp]
        h.oracle_closure_eval.argtypes = [i32, i32, i64, vp, vp, vp, vp, vp, vp, vp]
        _lib = h
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def _cfg(cfg):
    return C.byref(cfg.to_c()) if hasattr(cfg, "to_c") else C.byref(cfg)


def f_dtype(cfg, prec: int):
    if prec == 64:
        return np.float64
    return np.uint16 if cfg.use_float16c else np.float32


def step(cfg, grid, prec: int, f_out, f_in, bc, flags, tau: float, is_even: bool = False, nthreads: int = 0):
    """One step of the oracle.  prec 32: float32 arithmetic (Float16C storage when configured);
    prec 64: float64 arithmetic and storage.  For esoteric pull pass f_out is f_in."""
    g = grid.to_c()
    lib().oracle_step(_cfg(cfg), C.byref(g), prec, _p(f_out), _p(f_in), _p(bc), _p(flags), float(tau),
                      int(bool(is_even)), int(nthreads))


def step_range(cfg, grid, prec: int, f_out, f_in, bc, flags, tau: float, is_even: bool, begin: int, end: int,
               nthreads: int = 0):
    """The step on the cells with index x + nx*(y + ny*z) in [begin, end) only."""
    g = grid.to_c()
    lib().oracle_step_range(_cfg(cfg), C.byref(g), prec, _p(f_out), _p(f_in), _p(bc), _p(flags), float(tau),
                            int(bool(is_even)), int(nthreads), int(begin), int(end))


def init(cfg, grid, prec: int, f, rho: float = 1.0, tau: float = 1.0, u=None, grad=None):
    g = grid.to_c()
    u64 = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
    g64 = None if grad is None else np.ascontiguousarray(grad, dtype=np.float64)
    lib().oracle_init(_cfg(cfg), C.byref(g), prec, _p(f), float(rho), float(tau), _p(u64), _p(g64))


def rho_u(cfg, grid, prec: int, f, bc, flags, after_odd: bool = False):
    N, D = grid.num_points, grid.D
    dt = np.float64 if prec == 64 else np.float32
    rho = np.empty(N, dtype=dt)
    u = np.empty(D * N, dtype=dt)
    g = grid.to_c()
    lib().oracle_rho_u(_cfg(cfg), C.byref(g), prec, _p(f), _p(bc), _p(flags), _p(rho), _p(u), int(bool(after_odd)))
    return rho.reshape(grid.shape), u.reshape((D,) + grid.shape)


def q_criterion(cfg, grid, prec: int, f, bc, flags, u, tau: float, after_odd: bool = False, fill=np.nan):
    """Q-criterion [nx, ny, nz] of the state f with velocity u ([D, nx, ny, nz], e.g. from
    rho_u); cells with a raw SOLID flag keep `fill`."""
    dt = np.float64 if prec == 64 else np.float32
    q = np.full(grid.num_points, fill, dtype=dt)
    u = np.ascontiguousarray(u, dtype=dt)
    g = grid.to_c()
    lib().oracle_q_criterion(_cfg(cfg), C.byref(g), prec, _p(f), _p(bc), _p(flags), _p(u), float(tau),
                             int(bool(after_odd)), _p(q))
    return q.reshape(grid.shape)


def links(cfg, grid, prec: int, f, force, ids, dirs, dists, method: int, compute_force: bool, q_clamp: float):
    g = grid.to_c()
    lib().oracle_links(_cfg(cfg), C.byref(g), prec, _p(f), _p(force), _p(ids), _p(dirs), _p(dists), len(ids),
                       int(method), int(bool(compute_force)), float(q_clamp))


def drag(cfg, grid, prec: int, force, f, flags, ids):
    g = grid.to_c()
    lib().oracle_drag(_cfg(cfg), C.byref(g), prec, _p(force), _p(f), _p(flags), _p(ids), len(ids))


def gather(cfg, grid, prec: int, f, after_odd: bool = False):
    """[Q, nx, ny, nz] populations the next step would load (no boundary treatment)."""
    dt = np.float64 if prec == 64 else np.float32
    out = np.empty(grid.Q * grid.num_points, dtype=dt)
    g = grid.to_c()
    lib().oracle_gather(_cfg(cfg), C.byref(g), prec, _p(f), _p(out), int(bool(after_odd)))
    return out.reshape((grid.Q,) + grid.shape)


def f16c_encode(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty(x.shape, dtype=np.uint16)
    lib().oracle_f16c_encode(_p(x), _p(out), x.size)
    return out


def f16c_decode(h: np.ndarray) -> np.ndarray:
    h = np.ascontiguousarray(h, dtype=np.uint16)
    out = np.empty(h.shape, dtype=np.float32)
    lib().oracle_f16c_decode(_p(h), _p(out), h.size)
    return out


def layout_offset(grid, x, y, z, k, K) -> int:
    g = grid.to_c()
    return int(lib().oracle_layout_offset(C.byref(g), x, y, z, k, K))


def stress_pairs(D: int) -> list[list[int]]:
    """The (alpha, beta) pairs of the stress components, in the order the step sums them."""
    out = np.zeros(12, dtype=np.int32)
    n = lib().oracle_stress_pairs(int(D), _p(out))
    return out[: 2 * n].reshape(n, 2).tolist()


def lattice(lattice_id: int):
    c = np.zeros(27 * 3, dtype=np.int32)
    w = np.zeros(27, dtype=np.float64)
    o = np.zeros(27, dtype=np.int32)
    Q = lib().oracle_lattice(lattice_id, _p(c), _p(w), _p(o))
    return c[: 3 * Q].reshape(Q, 3), w[:Q], o[:Q]


def max_threads() -> int:
    return int(lib().oracle_max_threads())


class closure_t(C.Structure):
    """lbm_closure_t of include/lbm_gb300.h."""
    _fields_ = [("w1", C.c_float * 256), ("b1", C.c_float * 32), ("w2", C.c_float * 1024), ("b2", C.c_float * 32),
                ("w3", C.c_float * 32), ("b3", C.c_float), ("nu_scale", C.c_float),
                ("feat_mean", C.c_float * 8), ("feat_scale", C.c_float * 8), ("feat_lo", C.c_float * 8),
                ("feat_hi", C.c_float * 8)]


def closure_struct(theta: np.ndarray, nu_scale: float, mean, scale, lo, hi) -> closure_t:
    """Packs the 1377 parameters (w1, b1, w2, b2, w3, b3) and the feature normalisation."""
    t = np.asarray(theta, dtype=np.float32).ravel()
    c = closure_t()
    o = 0
    for name, n in (("w1", 256), ("b1", 32), ("w2", 1024), ("b2", 32), ("w3", 32)):
        getattr(c, name)[:] = t[o:o + n].tolist()
        o += n
    c.b3 = float(t[o])
    c.nu_scale = float(nu_scale)
    for name, v in (("feat_mean", mean), ("feat_scale", scale), ("feat_lo", lo), ("feat_hi", hi)):
        getattr(c, name)[:] = [float(a) for a in np.asarray(v, dtype=np.float64).ravel()]
    return c


def set_closure(c: closure_t | None) -> None:
    """Learned closure for the oracle's LES steps (None: Smagorinsky)."""
    lib().oracle_set_closure(None if c is None else C.byref(c))


def closure_eval(D: int, prec: int, S, s2, rho, uu, tau):
    """Features (n, 8) and nu_t (n; -1 outside the training range) for explicit strain rows."""
    S = np.ascontiguousarray(S, dtype=np.float64)
    n = S.shape[0]
    args = [np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (n,))) for a in (s2, rho, uu, tau)]
    x = np.zeros((n, 8), dtype=np.float64)
    nu = np.zeros(n, dtype=np.float64)
    lib().oracle_closure_eval(D, prec, n, _p(S), *[_p(a) for a in args], _p(x), _p(nu))
    return x, nu
