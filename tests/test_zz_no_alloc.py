"""The allocation-free mass/momentum reduction, lbm_reduce_mass_momentum_noalloc.

It exists for callers that cannot allocate device memory (their device memory comes from a pool
they do not own, or they run where cudaMalloc/cudaFree must not be called); it needs no handle
and keeps its scratch in a fixed device array inside the library.  This file is collected last so
that a run stopping at the first failure has run every other test first.  Each check calls the
entry point through the C ABI and compares it with lbm_reduce_mass_momentum (the handle-based
entry point) on the same populations: both reduce in float64 but in different block orders, so
they agree to a relative 1e-12.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from mojo_lbm_gb300 import LBM_Config, LBM_method, _capi
from mojo_lbm_gb300.solver import Solver
from tests.lbm_cases import initial_f, ldc_flags, make_grid

pytestmark = pytest.mark.gpu


def noalloc(cfg, grid, f, flags, after_odd: bool):
    out = (C.c_double * 4)()
    c, g = cfg.to_c(), grid.to_c()
    _capi.check(_capi.lib().lbm_reduce_mass_momentum_noalloc(C.byref(c), C.byref(g), f.data_ptr(), flags.data_ptr(),
                                                             int(after_odd), out, None))
    return np.array(out[:])


# every lattice x storage x streaming method appears; the cell counts are not multiples of 4096
# (the entry point's block), so each case's last block is partly filled
CASES = [("D3Q19", (56, 48, 40), (8, 8, 4), LBM_method.DOUBLE_BUFFER, False),
         ("D2Q9", (96, 80, 1), (16, 16, 1), LBM_method.ESOTERIC_PULL, True),
         ("D3Q27", (40, 24, 20), (8, 8, 4), LBM_method.ESOTERIC_PULL, False),
         ("D3Q19", (40, 24, 20), (8, 8, 4), LBM_method.ESOTERIC_PULL, True),
         ("D2Q9", (112, 48, 1), (16, 16, 1), LBM_method.DOUBLE_BUFFER, False),
         ("D3Q27", (24, 16, 40), (8, 8, 4), LBM_method.DOUBLE_BUFFER, True)]


def _case(lat, shape, tile, meth, f16, seed):
    grid = make_grid(lat, shape, tile)
    cfg = LBM_Config(meth, DDF_shift=f16, use_float16c=f16)
    flags, bc = ldc_flags(grid, cfg, 0.1)
    f0 = initial_f(grid, cfg, np.random.default_rng(seed), amp=0.04)
    f = torch.from_numpy(f0.view(np.int16) if f16 else f0).cuda()
    fl = torch.from_numpy(flags).cuda()
    return grid, cfg, f, fl


def test_noalloc_matches_handle_reduction_twice_in_a_row():
    """Six grids one after the other, each reduced twice in a row: no call may see the partials
    an earlier call left in the shared array."""
    for i, (lat, shape, tile, meth, f16) in enumerate(CASES):
        assert (shape[0] * shape[1] * shape[2]) % 4096 != 0
        grid, cfg, f, fl = _case(lat, shape, tile, meth, f16, 31 + i)
        ref = np.array(Solver(grid, cfg).mass_momentum(f, fl, after_odd_step=True))
        for _ in range(2):
            got = noalloc(cfg, grid, f, fl, True)
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-9 * abs(ref[0]))


def test_noalloc_at_its_maximum_size():
    """A grid of exactly 2^27 cells (the most the fixed scratch covers) is accepted and matches the
    handle-based reduction.  D2Q9 Float16C, periodic, from a rest equilibrium set on the device."""
    grid = make_grid("D2Q9", (16384, 8192, 1), (16, 16, 1))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, DDF_shift=True, use_float16c=True)
    f = torch.empty(grid.num_points * grid.Q, dtype=torch.int16, device="cuda")
    fl = torch.zeros(grid.num_points, dtype=torch.uint8, device="cuda")
    s = Solver(grid, cfg)
    s.init_equilibrium(f)
    ref = np.array(s.mass_momentum(f, fl))
    s.close()
    got = noalloc(cfg, grid, f, fl, False)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-9 * abs(ref[0]))
    assert ref[0] == pytest.approx(grid.num_points, rel=1e-6)


def test_noalloc_rejects_grids_beyond_its_scratch():
    grid = make_grid("D3Q19", (1024, 512, 512))      # 2^28 cells > 2^27
    c, g = LBM_Config().to_c(), grid.to_c()
    out = (C.c_double * 4)()
    st = _capi.lib().lbm_reduce_mass_momentum_noalloc(C.byref(c), C.byref(g), None, None, 0, out, None)
    assert st == _capi.LBM_EINVAL
    assert b"scratch covers at most" in _capi.lib().lbm_last_error()
