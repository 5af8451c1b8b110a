"""Checkpoint and resume: N steps equal N/2 steps, a save, a load and N/2 more, bit for bit — in
the float32 oracle (CPU) and through the library (GPU), for both streaming methods."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from mojo_lbm_gb300 import LBM_Config, LBM_method, checkpoint
from tests.lbm_cases import initial_f, ldc_flags, make_grid


def _oracle_steps(cfg, grid, f, f2, bc, flags, tau, k0, n):
    for k in range(k0, k0 + n):
        if cfg.lbm_method == LBM_method.DOUBLE_BUFFER:
            src, dst = (f, f2) if k % 2 == 0 else (f2, f)
            oracle.step(cfg, grid, 32, dst, src, bc, flags, tau)
        else:
            oracle.step(cfg, grid, 32, f, f, bc, flags, tau, k % 2 == 0)


@pytest.mark.parametrize("meth", ["db", "eso"])
def test_resume_is_exact_in_the_oracle(tmp_path, meth):
    grid = make_grid("D3Q19", (16, 8, 8), (8, 4, 4))
    m = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    cfg = LBM_Config(m, DDF_shift=True, use_float16c=True)
    flags, bc = ldc_flags(grid, cfg, 0.1)
    f0 = initial_f(grid, cfg, np.random.default_rng(1))
    a, a2 = f0.copy(), f0.copy()
    _oracle_steps(cfg, grid, a, a2, bc, flags, 0.7, 0, 10)
    b, b2 = f0.copy(), f0.copy()
    _oracle_steps(cfg, grid, b, b2, bc, flags, 0.7, 0, 5)
    p = checkpoint.save(tmp_path / "run", grid, cfg, f=b, f2=b2 if meth == "db" else None, bc=bc, flags=flags,
                        step=5, tau=0.7)
    d = checkpoint.load(p, grid, cfg)
    assert d["header"]["step"] == 5 and d["header"]["next_reads"] == "f2"
    c, c2 = d["f"].copy(), (d["f2"].copy() if d["f2"] is not None else d["f"].copy())
    _oracle_steps(cfg, grid, c, c2, d["bc"], d["flags"], d["header"]["tau"], d["header"]["step"], 5)
    assert np.array_equal(a, c) and (meth == "eso" or np.array_equal(a2, c2))


def test_load_rejects_a_different_layout(tmp_path):
    grid = make_grid("D3Q19", (16, 8, 8), (8, 4, 4))
    cfg = LBM_Config()
    flags, bc = ldc_flags(grid, cfg, 0.1)
    p = checkpoint.save(tmp_path / "x.npz", grid, cfg, f=np.zeros(grid.num_points * 19, np.float32), bc=bc,
                        flags=flags, step=0, tau=1.0)
    with pytest.raises(ValueError, match="grid"):
        checkpoint.load(p, make_grid("D3Q19", (16, 8, 8), (4, 4, 4)), cfg)
    with pytest.raises(ValueError, match="use_float16c"):
        checkpoint.load(p, grid, LBM_Config(use_float16c=True))


@pytest.mark.gpu
@pytest.mark.parametrize("meth", ["db", "eso"])
def test_resume_is_exact_on_the_gpu(tmp_path, meth):
    import torch

    from mojo_lbm_gb300.solver import Solver
    from tests.test_gpu_step import to_dev
    grid = make_grid("D3Q19", (32, 32, 16), (8, 8, 4))
    m = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    cfg = LBM_Config(m, LES=True)
    flags, bc = ldc_flags(grid, cfg, 0.1)
    f0 = initial_f(grid, cfg, np.random.default_rng(2))
    s = Solver(grid, cfg)
    a, a2 = to_dev(f0), to_dev(f0)
    bct, flt = to_dev(bc), to_dev(flags)
    s.run(a, a2, bct, flt, 0.6, 130, 0)  # one 64-step graph replay and 66 more
    b, b2 = to_dev(f0), to_dev(f0)
    s.run(b, b2, bct, flt, 0.6, 65, 0)
    p = checkpoint.save(tmp_path / "run", grid, cfg, f=b, f2=b2 if meth == "db" else None, bc=bct, flags=flt,
                        step=65, tau=0.6)
    d = checkpoint.load(p, grid, cfg, device="cuda")
    c = d["f"]
    c2 = d["f2"] if d["f2"] is not None else c
    s.run(c, c2, d["bc"], d["flags"], d["header"]["tau"], 65, d["header"]["step"])
    torch.cuda.synchronize()
    assert torch.equal(a, c) and (meth == "eso" or torch.equal(a2, c2))
