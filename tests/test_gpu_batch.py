"""The batched persistent step equals the single-domain step bit for bit: a batch of channels of
different sizes (moving-wall inlet, equilibrium outlet, cylinder with Bouzidi links) run by one
persistent launch per step, against each domain run alone through Solver (whose parity with the
oracle the other GPU tests establish)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from mojo_lbm_gb300 import Bounceback_method, LBM_Config, LBM_method
from mojo_lbm_gb300.batch import BatchSolver
from mojo_lbm_gb300.solver import Solver
from mojo_lbm_gb300.workloads import Channel, links_of

pytestmark = pytest.mark.gpu

SIZES = [(64, 32), (96, 48), (48, 16), (128, 48), (80, 32)]


def _channels():
    rng = np.random.default_rng(3)
    return [Channel(nx, ny, float(rng.uniform(20, 200)), 0.05, float(rng.uniform(-0.05, 0.05))) for nx, ny in SIZES]


def _f0(ch, cfg):
    f = torch.zeros(ch.grid.num_points * 9, device="cuda")
    s = Solver(ch.grid, cfg)
    u = torch.from_numpy(np.random.default_rng(5).uniform(-0.02, 0.02, (2,) + ch.grid.shape).astype(np.float32)).cuda()
    s.init_equilibrium(f, 1.0, ch.tau, u)
    if cfg.use_float16c:
        from mojo_lbm_gb300 import _capi
        h = torch.empty(f.numel(), dtype=torch.int16, device="cuda")
        _capi.check(_capi.lib().lbm_float16c_encode(f.data_ptr(), h.data_ptr(), f.numel(), None))
        return h
    return f


@pytest.mark.parametrize("variant", ["db-srt-links", "eso-trt", "db-kbc-f16c-links"])
def test_batch_equals_single_domain_steps(variant):
    chans = _channels()
    if variant == "db-srt-links":
        cfg = chans[0].cfg
    elif variant == "eso-trt":
        cfg = LBM_Config(LBM_method.ESOTERIC_PULL, collision_op="TRT", BCs={2}, DDF_shift=True)
    else:
        cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, collision_op="KBC", BCs={2}, DDF_shift=True, use_float16c=True)
    links = variant.endswith("links")
    steps = 70  # one 64-step graph replay + 6 direct steps
    batch = BatchSolver([c.grid for c in chans], cfg)
    bufs = []
    for i, ch in enumerate(chans):
        fa = _f0(ch, cfg)
        fb = fa.clone()
        bc = torch.from_numpy(ch.bc).cuda()
        fl = torch.from_numpy(ch.flags).cuda()
        bufs.append((fa, fb, bc, fl))
        batch.set_domain(i, fa, fb, bc, fl, ch.tau)
    ref = [(a.clone(), b.clone()) for a, b, _, _ in bufs]
    if links:
        dom, ids, dirs, dists, method = links_of(chans)
        batch.set_links(dom, ids, dirs, dists, method, 0.0)
    batch.run(steps, 0)
    for i, ch in enumerate(chans):
        s = Solver(ch.grid, cfg)
        fa, fb = ref[i]
        bc, fl = bufs[i][2], bufs[i][3]
        if links:
            ids = torch.from_numpy(ch.body.fluid_boundaries_list).cuda()
            dirs = torch.from_numpy(ch.body.lattice_links_list).cuda()
            dists = torch.from_numpy(ch.body.link_distances_list).cuda()
        for k in range(steps):
            if cfg.lbm_method == LBM_method.ESOTERIC_PULL:
                s.esoteric_pull_step(fa, bc, fl, ch.tau, k % 2 == 0)
                continue
            src, dst = (fa, fb) if k % 2 == 0 else (fb, fa)
            s.double_buffer_step(dst, src, bc, fl, ch.tau)
            if links:
                s.linkwise_bounceback(dst, None, ids, dirs, dists, Bounceback_method.BOUZIDI, False, 0.0)
        torch.cuda.synchronize()
        got_a, got_b = bufs[i][0], bufs[i][1]
        assert torch.equal(got_a, fa), f"domain {i} lattice A differs"
        assert torch.equal(got_b, fb), f"domain {i} lattice B differs"


def test_batch_full_size_equals_single_domain_steps():
    """The batched benchmark configuration at its full size: 512 channels (61 M cells, sizes on a
    32-cell granule, 32 x 8 tiles, Bouzidi links on every cylinder), one 64-step graph replay and
    two direct steps, against each channel stepped alone."""
    from mojo_lbm_gb300.workloads import channel_specs, cylinder_channels
    chans = cylinder_channels(tile=(32, 8, 1), specs=channel_specs(512, 0, granule=(32, 32)))
    assert sum(c.grid.num_points for c in chans) > 60_000_000
    cfg = chans[0].cfg
    steps = 66
    batch = BatchSolver([c.grid for c in chans], cfg)
    gen = torch.Generator(device="cuda").manual_seed(7)
    solvers, bufs, ref = [], [], []
    for i, ch in enumerate(chans):
        s = Solver(ch.grid, cfg)
        fa = torch.empty(ch.grid.num_points * 9, device="cuda")
        u = torch.empty((2,) + ch.grid.shape, device="cuda").uniform_(-0.02, 0.02, generator=gen)
        s.init_equilibrium(fa, 1.0, ch.tau, u)
        fb = fa.clone()
        bc = torch.from_numpy(ch.bc).cuda()
        fl = torch.from_numpy(ch.flags).cuda()
        batch.set_domain(i, fa, fb, bc, fl, ch.tau)
        solvers.append(s)
        bufs.append((fa, fb, bc, fl))
        ref.append((fa.clone(), fb.clone()))
    batch.set_links(*links_of(chans), 0.0)
    batch.run(steps, 0)
    for i, ch in enumerate(chans):
        s, (fa, fb), (_, _, bc, fl) = solvers[i], ref[i], bufs[i]
        ids = torch.from_numpy(ch.body.fluid_boundaries_list).cuda()
        dirs = torch.from_numpy(ch.body.lattice_links_list).cuda()
        dists = torch.from_numpy(ch.body.link_distances_list).cuda()
        for k in range(steps):
            src, dst = (fa, fb) if k % 2 == 0 else (fb, fa)
            s.double_buffer_step(dst, src, bc, fl, ch.tau)
            s.linkwise_bounceback(dst, None, ids, dirs, dists, Bounceback_method.BOUZIDI, False, 0.0)
    torch.cuda.synchronize()
    for i in range(len(chans)):
        assert torch.equal(bufs[i][0], ref[i][0]), f"domain {i} lattice A differs"
        assert torch.equal(bufs[i][1], ref[i][1]), f"domain {i} lattice B differs"


def test_batch_rejects_unsupported_tiles():
    from mojo_lbm_gb300 import LBM_Grid, get_D2Q9
    with pytest.raises(Exception, match="256-cell"):
        BatchSolver([LBM_Grid(get_D2Q9(), 30, 20, 1, (10, 5, 1))], LBM_Config())


def test_batch_flags_changing_between_runs():
    """Flags rewritten in place between batched runs (a block of SOLID cells appears in one
    channel, then the original flags return): the batch's warp masks follow each change, and the
    batch still equals the single-domain steps bit for bit."""
    chans = _channels()
    cfg = chans[0].cfg
    batch = BatchSolver([c.grid for c in chans], cfg)
    bufs = []
    for i, ch in enumerate(chans):
        fa = _f0(ch, cfg)
        bufs.append((fa, fa.clone(), torch.from_numpy(ch.bc).cuda(), torch.from_numpy(ch.flags).cuda()))
        batch.set_domain(i, *bufs[i], ch.tau)
    ref = [(a.clone(), b.clone()) for a, b, _, _ in bufs]
    solvers = [Solver(ch.grid, cfg) for ch in chans]
    blocked = chans[2].flags.copy()
    blocked[300:340] = 1  # SOLID cells in the interior of the third channel (its second tile)
    T, K = 256, 3  # the block's boundary values (read by the moving wall at a SOLID cell) are numbers
    cells = np.arange(300, 340)
    assert np.isfinite(chans[2].bc[(cells % T)[:, None] + T * (np.arange(K) + K * (cells // T)[:, None])]).all()
    plan = [(None, 3), (blocked, 4), (None, 64), (blocked, 1)]
    k = 0
    for new_flags, n in plan:
        bufs[2][3].copy_(torch.from_numpy(chans[2].flags if new_flags is None else new_flags))
        batch.run(n, k)
        for i, ch in enumerate(chans):
            fa, fb = ref[i]
            for j in range(n):
                src, dst = (fa, fb) if (k + j) % 2 == 0 else (fb, fa)
                solvers[i].double_buffer_step(dst, src, bufs[i][2], bufs[i][3], ch.tau)
        k += n
    torch.cuda.synchronize()
    for i in range(len(chans)):
        assert torch.equal(bufs[i][0], ref[i][0]) and torch.equal(bufs[i][1], ref[i][1]), f"domain {i} differs"
