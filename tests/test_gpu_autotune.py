"""The autotuner on the device: it times every candidate and returns one of them, for both
streaming methods when asked; a grid no candidate divides is reported, not guessed."""
from __future__ import annotations

import pytest

from mojo_lbm_gb300 import LBMError, LBM_Config, LBM_method, autotune, get_D2Q9, get_D3Q19

pytestmark = pytest.mark.gpu


def test_best_tile_is_a_candidate():
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER)
    tile, method, mlups = autotune.best_tile(cfg, get_D3Q19(), 64, 64, 32, steps=20)
    assert tile in autotune.candidates(get_D3Q19(), 64, 64, 32)
    assert method == LBM_method.DOUBLE_BUFFER and mlups > 0


def test_best_tile_chooses_method_and_caches():
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, use_float16c=True, DDF_shift=True)
    r1 = autotune.best_tile(cfg, get_D2Q9(), 512, 256, 1, choose_method=True, steps=20)
    assert r1[1] in (LBM_method.DOUBLE_BUFFER, LBM_method.ESOTERIC_PULL)
    assert autotune.best_tile(cfg, get_D2Q9(), 512, 256, 1, choose_method=True, steps=20) is r1


def test_untileable_grid_is_reported():
    with pytest.raises(LBMError, match="no 256-cell"):
        autotune.best_tile(LBM_Config(), get_D3Q19(), 30, 30, 30, steps=5)


def test_walled_domain_is_tuned_on_its_own_flags():
    """Timed on a cavity's flags the tuner avoids the long tiles a periodic box favours (they touch
    a wall almost everywhere and lose the all-fluid fast path)."""
    import numpy as np
    import torch

    from mojo_lbm_gb300 import LBM_Grid
    from tests.lbm_cases import ldc_flags
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER)
    grid = LBM_Grid(get_D3Q19(), 128, 128, 128)  # untiled layout
    flags, bc = ldc_flags(grid, cfg, 0.1)
    tile, _, _ = autotune.best_tile(cfg, get_D3Q19(), 128, 128, 128, flags=torch.from_numpy(flags).cuda(),
                                    bc=torch.from_numpy(bc).cuda(), key="cavity128", steps=30)
    assert tile in autotune.candidates(get_D3Q19(), 128, 128, 128)
    assert max(tile) <= 32, tile
