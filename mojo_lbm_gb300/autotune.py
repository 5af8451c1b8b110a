"""Autotuner front end: the tile shape of the layout (and optionally the streaming method) for a
configuration and grid size, chosen by timing on the device (``lbm_autotune``), cached per
process.  The tile is a layout choice, so it is made before the grid's buffers are allocated:

    tile, method, mlups = autotune.best_tile(cfg, get_D3Q19(), 256, 256, 256)
    grid = LBM_Grid(get_D3Q19(), 256, 256, 256, tile)
"""
from __future__ import annotations

import ctypes as C

from . import _capi
from ._capi import check

_cache: dict = {}


def candidates(lattice, nx: int, ny: int, nz: int) -> list[tuple[int, int, int]]:
    """The 256-cell power-of-two tiles dividing the grid (host only)."""
    lib = _capi.lib()
    n = lib.lbm_tune_candidates(lattice.id, nx, ny, nz, None, 0)
    if n < 0:
        raise ValueError("bad lattice or grid shape")
    buf = (C.c_int32 * (3 * max(n, 1)))()
    lib.lbm_tune_candidates(lattice.id, nx, ny, nz, buf, n)
    return [(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]) for i in range(n)]


def best_tile(config, lattice, nx: int, ny: int, nz: int, *, flags=None, bc=None, key=None,
              choose_method: bool = False, steps: int = 100, stream=None):
    """(tile, lbm_method, MLUPs) of the fastest candidate.

    flags / bc: the domain's device tensors in the untiled layout (an ``LBM_Grid`` with the default
    ``tile_shape="untiled"``), timed as they are; None times a periodic box of fluid.  Results are
    cached per (configuration, lattice, shape, choose_method, key) for the life of the process;
    pass a key naming the flag field when flags are given."""
    c = config.to_c()
    ck = (bytes(c), lattice.id, nx, ny, nz, bool(choose_method), key if flags is not None else None)
    if flags is not None and key is None:
        ck = None  # an unnamed flag field is not cached
    if ck is None or ck not in _cache:
        r = _capi.lbm_tune_result_t()
        check(_capi.lib().lbm_autotune(C.byref(c), lattice.id, nx, ny, nz, _capi.ptr(flags), _capi.ptr(bc),
                                       int(bool(choose_method)), int(steps), C.byref(r), _capi.stream_ptr(stream)))
        res = ((r.tx, r.ty, r.tz), r.lbm_method, float(r.mlups))
        if ck is None:
            return res
        _cache[ck] = res
    return _cache[ck]


def batch_tile(shapes, build, *, steps: int = 50, stream=None, samples: int = 4):
    """Tile for a batch of domains of one lattice and configuration: the candidates that divide
    every shape, each timed as a batch of about the same total size made of replicas of `samples`
    domains at evenly spaced quantiles of the size distribution (one persistent launch per step,
    graph-replayed).  Every replica has its own copy of its domain's flags and boundary values, so
    their reads cost what they cost in the real batch.  build(shape, tile) returns (grid, config,
    flags, bc, tau, links) with host arrays in that tile's layout, links None or (fluid ids,
    directions, distances) for Bouzidi bounce-back.  Returns (tile, {tile: MLUPs})."""
    import numpy as np
    import torch

    from .batch import BatchSolver
    from .constants import Bounceback_method
    from .solver import Solver
    shapes = [tuple(int(v) for v in s) for s in shapes]
    cells = np.array([int(np.prod(s)) for s in shapes])
    order = np.argsort(cells, kind="stable")
    k = max(1, min(int(samples), len(shapes)))
    picks = [shapes[int(order[int((2 * i + 1) * len(shapes) // (2 * k))])] for i in range(k)]
    reps = [max(1, int(round(cells.sum() / k / np.prod(p)))) for p in picks]
    grid0 = build(picks[0], picks[0])[0]
    common = None
    for s in shapes:
        c = set(candidates(grid0.lattice, *s))
        common = c if common is None else common & c
    if not common:
        raise ValueError("no 256-cell power-of-two tile divides every domain")
    timing = {}
    for tile in sorted(common):
        built = [build(p, tile) for p in picks]
        cfg = built[0][1]
        grids = [b[0] for b, r in zip(built, reps) for _ in range(r)]
        batch = BatchSolver(grids, cfg)
        dtype = torch.int16 if cfg.use_float16c else torch.float32
        keep, links_all = [], []
        i = 0
        for (grid, _, flags, bc, tau, links), r in zip(built, reps):
            f0 = torch.empty(grid.num_points * grid.Q, dtype=dtype, device="cuda")
            Solver(grid, cfg).init_equilibrium(f0)
            fl, b = torch.from_numpy(flags).cuda(), torch.from_numpy(bc).cuda()
            for _ in range(r):
                bufs = (f0.clone(), f0.clone(), b.clone(), fl.clone())
                keep.append(bufs)
                batch.set_domain(i, bufs[0], bufs[1], bufs[2], bufs[3], tau)
                if links is not None:
                    links_all.append((i, *(np.asarray(a) for a in links)))
                i += 1
        if links_all:
            t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).cuda()  # noqa: E731
            batch.set_links(t(np.concatenate([np.full(len(l[1]), l[0]) for l in links_all]), np.int32),
                            t(np.concatenate([l[1] for l in links_all]), np.int32),
                            t(np.concatenate([l[2] for l in links_all]), np.int32),
                            t(np.concatenate([l[3] for l in links_all]), np.float32),
                            Bounceback_method.BOUZIDI, 0.0)
        batch.run(64, 0, stream)
        cur = torch.cuda.current_stream() if stream is None else stream
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(cur)
        batch.run(steps, 0, stream)
        e1.record(cur)
        e1.synchronize()
        timing[tile] = sum(g.num_points for g in grids) * steps / (e0.elapsed_time(e1) * 1e-3) / 1e6
        batch.close()
        del keep
        torch.cuda.empty_cache()
    return max(timing, key=timing.get), timing
