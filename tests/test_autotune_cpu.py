"""The autotuner's candidate tiles (host only, no GPU): 256-cell power-of-two tiles dividing the
grid, 2D tiles flat in z."""
from __future__ import annotations

import pytest

from mojo_lbm_gb300 import autotune, get_D2Q9, get_D3Q19, get_D3Q27


def test_candidates_3d():
    c = autotune.candidates(get_D3Q19(), 256, 256, 256)
    assert (8, 8, 4) in c and (16, 16, 1) in c and (1, 1, 256) in c
    assert all(tx * ty * tz == 256 for tx, ty, tz in c)
    assert len(c) == len(set(c)) == 45  # (a, b, c) with a + b + c = 8: C(10, 2)


def test_candidates_respect_divisibility():
    c = autotune.candidates(get_D3Q27(), 64, 32, 8)
    assert c and all(64 % tx == 0 and 32 % ty == 0 and 8 % tz == 0 for tx, ty, tz in c)
    assert (4, 8, 8) in c and (8, 4, 8) in c and (16, 16, 1) in c
    assert autotune.candidates(get_D3Q19(), 30, 30, 30) == []


def test_candidates_2d():
    c = autotune.candidates(get_D2Q9(), 256, 96, 1)
    assert all(tz == 1 and tx * ty == 256 for tx, ty, tz in c)
    assert (16, 16, 1) in c and (32, 8, 1) in c and (256, 1, 1) in c and (8, 32, 1) in c
    assert (1, 256, 1) not in c  # 96 is not a multiple of 256


def test_candidates_reject_bad_shapes():
    with pytest.raises(ValueError):
        autotune.candidates(get_D2Q9(), 64, 64, 4)
    with pytest.raises(ValueError):
        autotune.candidates(get_D3Q19(), 0, 64, 64)


def test_channel_sizes_on_a_granule_admit_every_tile_of_the_granule():
    from mojo_lbm_gb300.workloads import channel_specs
    specs = channel_specs(64, seed=1, granule=(32, 32))
    common = None
    for nx, ny, Re, off in specs:
        assert nx % 32 == 0 and ny % 32 == 0 and 20 <= Re <= 200 and abs(off) <= 0.05
        c = set(autotune.candidates(get_D2Q9(), nx, ny, 1))
        common = c if common is None else common & c
    assert {(8, 32, 1), (16, 16, 1), (32, 8, 1)} <= common
