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


def batch_tile(shapes, build, *, steps: int = 50, stream=None):
    """Tile for a batch of domains of one lattice and configuration: the candidates that divide
    every shape, each timed as a batch of the same total size made of replicas of the median-size
    domain (one persistent launch per step, graph-replayed; the replicas share the domain's
    read-only flags and boundary arrays).  build(shape, tile) returns (grid, config, flags, bc,
    tau, links) with host arrays in that tile's layout, links None or (fluid ids, directions,
    distances) for Bouzidi bounce-back.  Returns (tile, {tile: MLUPs})."""
    import numpy as np
    import torch

    from .batch import BatchSolver
    from .constants import Bounceback_method
    from .solver import Solver
    shapes = [tuple(int(v) for v in s) for s in shapes]
    cells = np.array([int(np.prod(s)) for s in shapes])
    rep = shapes[int(np.argsort(cells)[len(cells) // 2])]
    replicas = max(1, int(round(cells.sum() / np.prod(rep))))
    grid0 = build(rep, rep)[0]
    common = None
    for s in shapes:
        c = set(candidates(grid0.lattice, *s))
        common = c if common is None else common & c
    if not common:
        raise ValueError("no 256-cell power-of-two tile divides every domain")
    timing = {}
    for tile in sorted(common):
        grid, cfg, flags, bc, tau, links = build(rep, tile)
        batch = BatchSolver([grid] * replicas, cfg)
        fl, b = torch.from_numpy(flags).cuda(), torch.from_numpy(bc).cuda()
        dtype = torch.int16 if cfg.use_float16c else torch.float32
        f0 = torch.empty(grid.num_points * grid.Q, dtype=dtype, device="cuda")
        Solver(grid, cfg).init_equilibrium(f0)
        bufs = []
        for i in range(replicas):
            fa, fb = f0.clone(), f0.clone()
            bufs.append((fa, fb))
            batch.set_domain(i, fa, fb, b, fl, tau)
        if links is not None:
            ids, dirs, dists = (np.asarray(a) for a in links)
            n = len(ids)
            t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).cuda()  # noqa: E731
            batch.set_links(t(np.repeat(np.arange(replicas), n), np.int32), t(np.tile(ids, replicas), np.int32),
                            t(np.tile(dirs, replicas), np.int32), t(np.tile(dists, replicas), np.float32),
                            Bounceback_method.BOUZIDI, 0.0)
        batch.run(64, 0, stream)
        cur = torch.cuda.current_stream() if stream is None else stream
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(cur)
        batch.run(steps, 0, stream)
        e1.record(cur)
        e1.synchronize()
        timing[tile] = replicas * grid.num_points * steps / (e0.elapsed_time(e1) * 1e-3) / 1e6
        batch.close()
        del bufs
        torch.cuda.empty_cache()
    return max(timing, key=timing.get), timing
