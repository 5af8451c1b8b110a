"""Interpolated bounce-back fused into the step (lbm_set_links) against the link-wise path it
replaces: the step, then the link-wise kernel (src/lbm/geometry/interpolated_BB.mojo:46-141) on the
lattice the step wrote.

The fused step applies at step k the links the link-wise path applies after step k-1 (its first
step, those of a link pass over the lattice it is given: the link-wise runs here start with one
over the initial state), so after K steps the two lattices differ only in the link slots (x, i);
one link-wise pass over the fused lattice closes that gap.  Float32 (exact arithmetic): every word
equal, and the link forces the fused step k writes equal the link-wise forces of step k-1.
Float16C: the link-wise path rounds the interpolated value to a 16-bit code before the next step
reads it and the fused path does not, so values agree to two units in the code's last place
(2^-9 |f|) plus an absolute 8e-6 (two code units of a population of magnitude 0.01, the scale of
the DDF-shifted populations, whose rounding difference the collision spreads to smaller
neighbours) after K steps.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from mojo_lbm_gb300 import Bounceback_method, Flags, LBM_Config, LBM_Grid, LBM_method, preprocess
from mojo_lbm_gb300.geometry import get_rigid_sphere
from mojo_lbm_gb300.lattice import get_lattice
from mojo_lbm_gb300.solver import Solver
from tests.lbm_cases import initial_f

pytestmark = pytest.mark.gpu

STEPS = 7


def _case(lat: str, f16: bool, arithmetic: str = "exact"):
    """A channel with no-slip walls on +-Y (the +Y wall moving), periodic along x (and z), and a
    cylinder (D2Q9) or a sphere (D3Q19, D3Q27) with its links; a seeded velocity field."""
    lid = {"D2Q9": 0, "D3Q19": 1, "D3Q27": 2}[lat]
    if lid == 0:
        grid = LBM_Grid(get_lattice(0), 64, 48, 1, (16, 16, 1))
        center, radius = (20.3, 23.6, 0.0), 7.3
    else:
        grid = LBM_Grid(get_lattice(lid), 32, 32, 16, (8, 8, 4))
        center, radius = (12.4, 15.7, 7.8), 4.6
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, DDF_shift=f16, use_float16c=f16, arithmetic=arithmetic)
    N, D = grid.num_points, grid.D
    flags, bc = np.zeros(N, np.uint8), np.zeros(N * (D + 1), np.float32)
    preprocess.set_exterior_walls(grid, cfg, flags, bc, "-Y", Flags.SOLID, [0.0] * D, 1.0)
    preprocess.set_exterior_walls(grid, cfg, flags, bc, "+Y", Flags.SOLID, [0.03] + [0.0] * (D - 1), 1.0)
    body = get_rigid_sphere(grid, flags, center, radius, device="cpu")
    f0 = initial_f(grid, cfg, np.random.default_rng(5 + lid), amp=0.03, tau=0.7)
    return grid, cfg, flags, bc, f0, body


def _dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a.view(np.int16) if a.dtype == np.uint16 else a)).cuda()


def _host(t: torch.Tensor, like: np.ndarray) -> np.ndarray:
    a = t.cpu().numpy()
    return a.view(np.uint16) if like.dtype == np.uint16 else a


def _links(body):
    t = lambda a, dt: torch.from_numpy(np.asarray(a).astype(dt)).cuda()  # noqa: E731
    return (t(body.fluid_boundaries_list, np.int32), t(body.lattice_links_list, np.int32),
            t(body.link_distances_list, np.float32))


def _run_linkwise(grid, cfg, flags, bc, f0, body, method, tau, steps):
    s = Solver(grid, cfg)
    fa, fb, bct, flt = _dev(f0), _dev(f0), _dev(bc), _dev(flags)
    ids, dirs, dists = _links(body)
    s.linkwise_bounceback(fa, None, ids, dirs, dists, method, False, 0.0)  # the links of the initial state
    forces = []
    for k in range(steps):
        src, dst = (fa, fb) if k % 2 == 0 else (fb, fa)
        s.double_buffer_step(dst, src, bct, flt, tau)
        force = torch.zeros(ids.numel() * grid.D, device="cuda")
        s.linkwise_bounceback(dst, force, ids, dirs, dists, method, True, 0.0)
        forces.append(force)
    torch.cuda.synchronize()
    out = fa if steps % 2 == 0 else fb
    res = _host(out, f0), [f.cpu().numpy() for f in forces]
    s.close()
    return res


def _run_fused(grid, cfg, flags, bc, f0, body, method, tau, steps, by_run=False):
    s = Solver(grid, cfg)
    assert s.kernel_path in (2, 3)
    fa, fb, bct, flt = _dev(f0), _dev(f0), _dev(bc), _dev(flags)
    ids, dirs, dists = _links(body)
    force = torch.zeros(ids.numel() * grid.D, device="cuda")
    s.set_links(ids, dirs, dists, method, 0.0, force)
    forces = []
    if by_run:
        s.run(fa, fb, bct, flt, tau, steps, 0)
    else:
        for k in range(steps):
            src, dst = (fa, fb) if k % 2 == 0 else (fb, fa)
            s.double_buffer_step(dst, src, bct, flt, tau)
            forces.append(force.clone())
    out = fa if steps % 2 == 0 else fb
    # one link-wise pass turns the fused lattice into the link-wise path's
    s.linkwise_bounceback(out, None, ids, dirs, dists, method, False, 0.0)
    torch.cuda.synchronize()
    res = _host(out, f0), [f.cpu().numpy() for f in forces]
    s.close()
    return res


def _close_f16(got, ref, what):
    g = oracle.f16c_decode(got).astype(np.float64)
    r = oracle.f16c_decode(ref).astype(np.float64)
    tol = 8e-6 + 2.0 ** -9 * np.abs(r)
    bad = ~(np.abs(g - r) <= tol)
    assert not bad.any(), f"{what}: {int(bad.sum())} values beyond the tolerance (max |df| {np.abs(g - r).max():.3e})"


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
@pytest.mark.parametrize("method", [Bounceback_method.BOUZIDI, Bounceback_method.MID_GRID])
@pytest.mark.parametrize("f16", [False, True])
def test_fused_links_match_linkwise(lat, method, f16):
    grid, cfg, flags, bc, f0, body = _case(lat, f16)
    assert body.num_links() > 50
    # both halves of the interpolation are exercised
    q = np.asarray(body.link_distances_list)
    assert (q > 0.5).any() and (q <= 0.5).any()
    ref, ref_forces = _run_linkwise(grid, cfg, flags, bc, f0, body, method, 0.7, STEPS)
    got, got_forces = _run_fused(grid, cfg, flags, bc, f0, body, method, 0.7, STEPS)
    if f16:
        _close_f16(got, ref, f"{lat} Float16C")
    else:
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), \
            f"{int((got.view(np.uint32) != ref.view(np.uint32)).sum())} words differ"
        for k in range(1, STEPS):  # the fused step k writes the link-wise forces of step k-1
            assert np.array_equal(got_forces[k].view(np.uint32), ref_forces[k - 1].view(np.uint32)), k


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19"])
def test_fused_links_graph_run(lat):
    """The same through lbm_run (64-step CUDA graph replays): 66 steps."""
    grid, cfg, flags, bc, f0, body = _case(lat, False)
    ref, _ = _run_linkwise(grid, cfg, flags, bc, f0, body, Bounceback_method.BOUZIDI, 0.7, 66)
    got, _ = _run_fused(grid, cfg, flags, bc, f0, body, Bounceback_method.BOUZIDI, 0.7, 66, by_run=True)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19"])
def test_fused_links_fast_arithmetic(lat):
    """The fast build with fused links tracks the exact link-wise path to its stated tolerance over
    a few steps (float32: 1e-6 + 2e-6 |f| per step, compounding)."""
    grid, cfg, flags, bc, f0, body = _case(lat, False, "fast")
    ref, _ = _run_linkwise(grid, LBM_Config(LBM_method.DOUBLE_BUFFER), flags, bc, f0, body,
                           Bounceback_method.BOUZIDI, 0.7, 3)
    got, _ = _run_fused(grid, cfg, flags, bc, f0, body, Bounceback_method.BOUZIDI, 0.7, 3)
    assert np.abs(got.astype(np.float64) - ref).max() <= 3 * (1e-6 + 2e-6 * np.abs(ref).max())


def test_set_links_rejects_bad_links():
    grid, cfg, flags, bc, f0, body = _case("D2Q9", False)
    s = Solver(grid, cfg)
    ids, dirs, dists = _links(body)
    for bad_ids, bad_dirs in ((ids.clone().fill_(grid.num_points), dirs), (ids, dirs.clone().fill_(0)),
                              (torch.cat([ids, ids[:1]]), torch.cat([dirs, dirs[:1]]))):
        d = dists if bad_ids.numel() == dists.numel() else torch.cat([dists, dists[:1]])
        with pytest.raises(Exception):
            s.set_links(bad_ids, bad_dirs, d, Bounceback_method.BOUZIDI)
    s.set_links(ids, dirs, dists, Bounceback_method.BOUZIDI)
    with pytest.raises(Exception):  # the fused links run in the block-per-tile kernel only
        s.set_kernel_path(1)
    s.set_links(None, None, None, Bounceback_method.BOUZIDI)  # removed: the generic kernel is allowed again
    s.set_kernel_path(1)
    s.close()


def test_batch_fused_links_match_separate():
    """Five cylinder channels of the batched workload: LBM_LINKS_FUSED (one kernel per step) against
    LBM_LINKS_SEPARATE (the link-wise kernel after every step), word for word after a final link
    pass, and the forces one step apart."""
    import oracle as orc
    from mojo_lbm_gb300.batch import BatchSolver
    from mojo_lbm_gb300.workloads import cylinder_channels, links_of
    chans = cylinder_channels(n=5, seed=3, nx_range=(96, 160), tile=(16, 16, 1))
    dom, ids, dirs, dists, method = links_of(chans)
    runs = {}
    for fused in (False, True):
        b = BatchSolver([c.grid for c in chans], chans[0].cfg)
        bufs = []
        for i, ch in enumerate(chans):
            f = np.zeros(ch.grid.num_points * 9, np.float32)
            orc.init(ch.cfg, ch.grid, 32, f)
            fa, fb = _dev(f), _dev(f)
            bct, flt = _dev(ch.bc), _dev(ch.flags)
            if not fused:  # the link-wise path starts from a link pass over the initial state
                s = Solver(ch.grid, ch.cfg)
                sel = (dom == i).nonzero().flatten()
                s.linkwise_bounceback(fa, None, ids[sel], dirs[sel], dists[sel], method, False, 0.0)
                torch.cuda.synchronize()
                s.close()
            bufs.append((fa, fb, bct, flt))
            b.set_domain(i, fa, fb, bct, flt, ch.tau)
        force = torch.zeros(ids.numel() * 2, device="cuda")
        b.set_links(dom, ids, dirs, dists, method, 0.0, force)
        b.set_link_mode(fused)
        b.run(STEPS - 1, 0)
        f_prev = force.clone()
        b.run(1, STEPS - 1)
        torch.cuda.synchronize()
        outs = []
        for i, ch in enumerate(chans):
            out = bufs[i][1] if STEPS % 2 == 1 else bufs[i][0]
            if fused:
                s = Solver(ch.grid, ch.cfg)
                sel = (dom == i).nonzero().flatten()
                s.linkwise_bounceback(out, None, ids[sel], dirs[sel], dists[sel], method, False, 0.0)
                torch.cuda.synchronize()
                s.close()
            outs.append(out.cpu().numpy())
        runs[fused] = (outs, f_prev.cpu().numpy(), force.cpu().numpy())
        b.close()
    (sep, sep_prev, _), (fus, _, fus_last) = runs[False], runs[True]
    for a, c in zip(sep, fus):
        assert np.array_equal(a.view(np.uint32), c.view(np.uint32))
    assert np.array_equal(fus_last.view(np.uint32), sep_prev.view(np.uint32))
