"""Assembly (the mirror of src/lbm/assembly.mojo:43-269) on the CPU: its buffers per method and
storage, the buffer views of each method, and wall painting into the host flags and bc (compared
with the oracle's restatement of the reference's painting) followed by the upload."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from mojo_lbm_gb300 import Flags, LBM_Config, LBM_method
from mojo_lbm_gb300.assembly import Assembly
from oracle import paint
from tests.lbm_cases import make_grid


@pytest.mark.parametrize("meth,f16", [(LBM_method.DOUBLE_BUFFER, False), (LBM_method.ESOTERIC_PULL, True)])
def test_buffers_and_views(meth, f16):
    grid = make_grid("D3Q19", (16, 16, 8), (8, 8, 4))
    cfg = LBM_Config(meth, DDF_shift=f16, use_float16c=f16)
    a = Assembly(grid, cfg, device="cpu")
    N, Q = grid.num_points, grid.Q
    assert a.f.numel() == N * Q and a.f.dtype == (torch.int16 if f16 else torch.float32)
    assert a.bc.numel() == N * 4 and a.bc.dtype == torch.float32
    assert a.flags.numel() == N and a.flags.dtype == torch.uint8
    if meth == LBM_method.DOUBLE_BUFFER:
        assert a.f2 is not None and a.f2.shape == a.f.shape
        f, f2, bc, fl = a.get_gpu_tensors_for_double_buffer()
        assert f is a.f and f2 is a.f2 and bc is a.bc and fl is a.flags
        with pytest.raises(RuntimeError, match="Esoteric Pull"):
            a.get_gpu_tensors_for_esoteric_pull()
    else:
        assert a.f2 is None
        f, bc, fl = a.get_gpu_tensors_for_esoteric_pull()
        assert f is a.f and bc is a.bc and fl is a.flags
        with pytest.raises(RuntimeError, match="Double Buffer"):
            a.get_gpu_tensors_for_double_buffer()


@pytest.mark.parametrize("lat,shape,tile", [("D2Q9", (32, 16, 1), (16, 16, 1)), ("D3Q27", (16, 8, 16), (4, 8, 8))])
def test_walls_paint_host_arrays_and_upload(lat, shape, tile):
    grid = make_grid(lat, shape, tile)
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, BCs={Flags.EQUILIBRIUM})
    a = Assembly(grid, cfg, device="cpu")
    D = grid.D
    lid = [0.1] + [0.0] * (D - 1)
    sides = [("-X", Flags.SOLID, [0.0] * D, 1.0), ("+X", Flags.EQUILIBRIUM, [], 1.0), ("+Y", Flags.SOLID, lid, 1.0)]
    if D == 3:
        sides.append(("-Z", Flags.SOLID, [0.0] * D, 1.0))
    flags = np.zeros(grid.num_points, np.uint8)
    bc = np.zeros(grid.num_points * (D + 1), np.float32)
    for side, kind, u, rho in sides:
        a.set_exterior_walls(side, kind, u, rho)
        vel = list(u) + [float("nan")] * (D - len(u))
        paint.paint_wall(shape, tile, D, flags, bc, side, kind, vel, rho)
    assert np.array_equal(a.flags_host, flags)
    assert np.array_equal(a.bc_host.view(np.uint32), bc.view(np.uint32))
    assert int(a.flags.sum()) == 0  # nothing on the device side before the upload
    a.upload()
    assert np.array_equal(a.flags.numpy(), flags)
    assert np.array_equal(a.bc.numpy().view(np.uint32), bc.view(np.uint32))


def test_wall_from_a_function():
    """set_exterior_walls with u_func: a parabolic inlet on -X, evaluated at the face's cells."""
    grid = make_grid("D2Q9", (32, 16, 1), (16, 16, 1))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER)
    a = Assembly(grid, cfg, device="cpu")
    H = grid.ny - 1.0
    a.set_exterior_walls("-X", Flags.SOLID, rho=1.0, u_func=lambda x, y, z: (0.2 * y * (H - y) / (H * H), 0.0 * y))
    flags = np.zeros(grid.num_points, np.uint8)
    bc = np.zeros(grid.num_points * 3, np.float32)
    y = np.arange(grid.ny, dtype=np.float64)
    u_face = [np.asarray(0.2 * y * (H - y) / (H * H), np.float32), np.zeros(grid.ny, np.float32)]
    paint.paint_wall_values((32, 16, 1), (16, 16, 1), 2, flags, bc, "-X", Flags.SOLID, u_face, 1.0)
    assert np.array_equal(a.flags_host, flags)
    assert np.array_equal(a.bc_host.view(np.uint32), bc.view(np.uint32))
