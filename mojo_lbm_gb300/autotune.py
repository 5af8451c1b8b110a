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
