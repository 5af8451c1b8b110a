"""GPU tests of everything around the step, through the C ABI, against the oracle, bit for bit
unless stated: Float16C codec, device initialisation, the graph-replayed time loop, rho/u
output, float64 mass/momentum reduction (summation order differs: relative 1e-12), link-wise
interpolated bounce-back with its force, and the drag force."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from mojo_lbm_gb300 import Bounceback_method, Flags, LBM_Config, LBM_method, _capi
from mojo_lbm_gb300.geometry import get_rigid_sphere
from mojo_lbm_gb300.solver import Solver
from tests.lbm_cases import initial_f, ldc_flags, make_grid, mixed_flags, random_velocity
from tests.test_gpu_step import assert_close, to_dev, to_host

pytestmark = pytest.mark.gpu


def test_codec_decode_all_codes_bit_exact():
    codes = np.arange(65536, dtype=np.uint16)
    d_in = to_dev(codes)
    d_out = torch.empty(65536, dtype=torch.float32, device="cuda")
    _capi.check(_capi.lib().lbm_float16c_decode(d_in.data_ptr(), d_out.data_ptr(), 65536, None))
    got = d_out.cpu().numpy().view(np.uint32)
    ref = oracle.f16c_decode(codes).view(np.uint32)
    assert np.array_equal(got, ref)


def test_codec_encode_bit_exact():
    rng = np.random.default_rng(0)
    x = np.concatenate([
        rng.normal(0, 1, 200000).astype(np.float32),
        (rng.normal(0, 1, 200000) * 10.0 ** rng.uniform(-12, 4, 200000)).astype(np.float32),
        np.array([0.0, -0.0, 1.0, -1.0, 1.999, 2.0, 65504.0, 1e-8, 3e-5, np.inf, -np.inf, np.nan], np.float32),
        rng.integers(0, 2 ** 32, 100000, dtype=np.uint64).astype(np.uint32).view(np.float32),
    ])
    d_in = torch.from_numpy(x).cuda()
    d_out = torch.empty(x.size, dtype=torch.int16, device="cuda")
    _capi.check(_capi.lib().lbm_float16c_encode(d_in.data_ptr(), d_out.data_ptr(), x.size, None))
    got = d_out.cpu().numpy().view(np.uint16)
    assert np.array_equal(got, oracle.f16c_encode(x))


@pytest.mark.parametrize("lat,meth,f16,grad", [("D2Q9", "db", False, True), ("D3Q19", "eso", False, True),
                                               ("D3Q27", "db", True, False), ("D3Q19", "eso", True, True)])
def test_init_equilibrium(lat, meth, f16, grad):
    shape = {"D2Q9": (20, 12, 1), "D3Q19": (12, 8, 6), "D3Q27": (8, 8, 6)}[lat]
    grid = make_grid(lat, shape, (4, 4, 1) if lat == "D2Q9" else (4, 4, 3))
    m = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    cfg = LBM_Config(m, DDF_shift=f16, use_float16c=f16)
    rng = np.random.default_rng(1)
    u = random_velocity(grid, rng).astype(np.float32)
    g = rng.normal(0, 1e-3, (grid.D * grid.D,) + grid.shape).astype(np.float32) if grad else None
    ref = np.zeros(grid.num_points * grid.Q, oracle.f_dtype(cfg, 32))
    oracle.init(cfg, grid, 32, ref, 1.0, 0.7, u, g)
    solver = Solver(grid, cfg)
    fd = torch.zeros(ref.size, dtype=torch.int16 if f16 else torch.float32, device="cuda")
    solver.init_equilibrium(fd, 1.0, 0.7, torch.from_numpy(u).cuda(),
                            None if g is None else torch.from_numpy(g).cuda())
    got = to_host(fd, ref)
    assert_close(got, ref, cfg, "init")


@pytest.mark.parametrize("meth", ["db", "eso"])
@pytest.mark.parametrize("n_steps,first", [(130, 0), (67, 1), (5, 0)])
def test_run_graph_matches_steps(meth, n_steps, first):
    """lbm_run (64-step graph replays + direct launches) equals the single-step calls bit for bit."""
    grid = make_grid("D3Q19", (16, 12, 8), (8, 4, 4))
    m = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    cfg = LBM_Config(m, DDF_shift=True)
    flags, bc = ldc_flags(grid, cfg, 0.05)
    f0 = initial_f(grid, cfg, np.random.default_rng(9))
    s = Solver(grid, cfg)
    bct, flt = to_dev(bc), to_dev(flags)
    a1, b1 = to_dev(f0), to_dev(f0)
    a2, b2 = to_dev(f0), to_dev(f0)
    s.run(a1, b1, bct, flt, 0.7, n_steps, first)
    for k in range(n_steps):
        par = (first + k) % 2 == 0
        if m == LBM_method.ESOTERIC_PULL:
            s.esoteric_pull_step(a2, bct, flt, 0.7, par)
        elif par:
            s.double_buffer_step(b2, a2, bct, flt, 0.7)
        else:
            s.double_buffer_step(a2, b2, bct, flt, 0.7)
    torch.cuda.synchronize()
    assert torch.equal(a1, a2) and torch.equal(b1, b2)


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
@pytest.mark.parametrize("meth", ["db", "eso"])
def test_rho_u_output(lat, meth):
    shape = {"D2Q9": (24, 16, 1), "D3Q19": (12, 8, 8), "D3Q27": (8, 8, 8)}[lat]
    grid = make_grid(lat, shape, (8, 8, 1) if lat == "D2Q9" else (4, 4, 4))
    m = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    cfg = LBM_Config(m, BCs={Flags.EQUILIBRIUM}, DDF_shift=True)
    rng = np.random.default_rng(4)
    flags, bc = mixed_flags(grid, rng)
    flags = np.where(flags & Flags.EXCLUDE, Flags.FLUID, flags).astype(np.uint8)
    f0 = initial_f(grid, cfg, rng)
    s = Solver(grid, cfg)
    rho = torch.empty(grid.num_points, device="cuda")
    u = torch.empty(grid.num_points * grid.D, device="cuda")
    for after_odd in ([False] if meth == "db" else [False, True]):
        s.compute_rho_u(rho, u, to_dev(f0), to_dev(bc), to_dev(flags), after_odd)
        r_ref, u_ref = oracle.rho_u(cfg, grid, 32, f0, bc, flags, after_odd)
        assert np.array_equal(rho.cpu().numpy().reshape(grid.shape), r_ref, equal_nan=True)
        assert np.array_equal(u.cpu().numpy().reshape((grid.D,) + grid.shape), u_ref, equal_nan=True)


@pytest.mark.parametrize("meth", ["db", "eso"])
def test_mass_momentum_conserved(meth):
    """Float64 mass of the populations the next step loads is conserved to float32 rounding:
    in a closed box with stationary walls (double buffer) and on a periodic box (esoteric pull,
    whose implicit bounce-back parks wall populations in solid slots for one step)."""
    grid = make_grid("D3Q19", (24, 24, 24), (8, 8, 8))
    m = LBM_method.DOUBLE_BUFFER if meth == "db" else LBM_method.ESOTERIC_PULL
    cfg = LBM_Config(m, include_moving_boundary=False)
    flags, bc = ldc_flags(grid, cfg, 0.0)
    if m == LBM_method.ESOTERIC_PULL:
        flags[:] = Flags.FLUID
    f0 = initial_f(grid, cfg, np.random.default_rng(2), amp=0.03, noise=0.0)
    s = Solver(grid, cfg)
    a, b = to_dev(f0), to_dev(f0)
    bct, flt = to_dev(bc), to_dev(flags)
    m0 = s.mass_momentum(a, flt, after_odd_step=True)
    ref = oracle.gather(cfg, grid, 32, f0, after_odd=True).astype(np.float64)
    fluid = (grid.layouts.from_layout(flags, 1)[..., 0] & 0x0F) != Flags.SOLID
    assert abs(m0[0] - ref.sum(0)[fluid].sum()) < 1e-6 * m0[0]
    s.run(a, b, bct, flt, 0.8, 200, 0)
    m1 = s.mass_momentum(a, flt, after_odd_step=True)
    assert abs(m1[0] - m0[0]) / m0[0] < 1e-5, (m0, m1)


def test_mass_reduction_reports_nan():
    grid = make_grid("D2Q9", (16, 16, 1))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER)
    f = torch.zeros(grid.num_points * 9, device="cuda")
    f[17] = float("nan")
    s = Solver(grid, cfg)
    with pytest.raises(_capi.LBMError) as e:
        s.mass_momentum(f, torch.zeros(grid.num_points, dtype=torch.uint8, device="cuda"))
    assert e.value.status == _capi.LBM_ENAN


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19"])
@pytest.mark.parametrize("method", [Bounceback_method.BOUZIDI, Bounceback_method.MID_GRID])
@pytest.mark.parametrize("f16", [False, True])
def test_linkwise_bounceback_and_force(lat, method, f16):
    shape = {"D2Q9": (48, 32, 1), "D3Q19": (24, 16, 16)}[lat]
    grid = make_grid(lat, shape, (8, 8, 1) if lat == "D2Q9" else (8, 8, 4))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, DDF_shift=f16, use_float16c=f16)
    flags = np.zeros(grid.num_points, np.uint8)
    center = [20.3, 15.7, 7.9 if lat == "D3Q19" else 0.0]
    obj = get_rigid_sphere(grid, flags, center, 6.2)
    assert obj.num_links() > 0
    f0 = initial_f(grid, cfg, np.random.default_rng(8))
    s = Solver(grid, cfg)
    fd = to_dev(f0)
    obj.bounceback(s, fd, method, True, 0.01)
    ids, dirs, dists = obj.fluid_boundaries_list, obj.lattice_links_list, obj.link_distances_list
    fr = f0.copy()
    force = np.zeros(len(ids) * grid.D, np.float32)
    oracle.links(cfg, grid, 32, fr, force, ids, dirs, dists, method, True, 0.01)
    assert_close(to_host(fd, f0), fr, cfg, "links")
    assert np.array_equal(obj.link_forces[: len(ids) * grid.D].cpu().numpy(), force)
    F = obj.sum_force(s)
    np.testing.assert_allclose(F, force.reshape(grid.D, -1).astype(np.float64).sum(1), rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q27"])
def test_drag_force(lat):
    shape = {"D2Q9": (40, 24, 1), "D3Q27": (16, 16, 12)}[lat]
    grid = make_grid(lat, shape, (8, 8, 1) if lat == "D2Q9" else (8, 8, 4))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, DDF_shift=True)
    flags = np.zeros(grid.num_points, np.uint8)
    obj = get_rigid_sphere(grid, flags, [17.2, 11.9, 5.5 if lat == "D3Q27" else 0.0], 4.7)
    ids = obj.unique_fluid_ids
    f0 = initial_f(grid, cfg, np.random.default_rng(12))
    s = Solver(grid, cfg)
    out = torch.empty(len(ids) * grid.D, device="cuda")
    s.drag_force(out, to_dev(f0), to_dev(flags), torch.from_numpy(ids).cuda())
    ref = np.zeros(len(ids) * grid.D, np.float32)
    oracle.drag(cfg, grid, 32, ref, f0, flags, ids)
    assert np.array_equal(out.cpu().numpy(), ref)


def test_errors_do_not_touch_device():
    grid = make_grid("D3Q19", (8, 8, 8))
    s = Solver(grid, LBM_Config(LBM_method.ESOTERIC_PULL))
    f = torch.zeros(grid.num_points * 19, device="cuda")
    with pytest.raises(_capi.LBMError):
        s.double_buffer_step(f, f, None, None, 0.8)
    with pytest.raises(_capi.LBMError) as e:
        s.linkwise_bounceback(f, None, torch.zeros(1, dtype=torch.int32, device="cuda"),
                              torch.zeros(1, dtype=torch.int32, device="cuda"), torch.zeros(1, device="cuda"), 1)
    assert e.value.status == _capi.LBM_EUNSUPPORTED
    assert _capi.lib().lbm_last_error()
