"""CPU checks of the oracle: the Ghia et al. cavity fixture the reference ships, Float16C
known answers, layout known answers, lattice tables, and the invariants of the step."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from mojo_lbm_gb300 import Flags, LBM_Config, LBM_method, get_D2Q9, get_D3Q19, get_D3Q27
from tests.conftest import needs_reference, reference_root
from tests.lbm_cases import initial_f, ldc_flags, make_grid, mixed_flags

GOLDEN = Path(__file__).with_name("golden")


# ---- Float16C (src/utils/custom_fp.mojo:36-101) -------------------------------------------
# Known answers derived by hand from the format: sign | 4-bit exponent (bias offset 112 from
# float32) | 11-bit mantissa.
F16C_KAT = [
    (0x0000, 0.0), (0x8000, -0.0), (0x7800, 1.0), (0xF800, -1.0), (0x7000, 2.0 ** -1),
    (0x0800, 2.0 ** -14), (0x7FFF, 2.0 - 2.0 ** -11), (0x7C00, 1.5), (0x0400, 2.0 ** -15),
    (0x0001, 2.0 ** -25), (0x3C00, 1.5 * 2.0 ** -8),
]


@pytest.mark.parametrize("code,value", F16C_KAT)
def test_f16c_known_answers(code, value):
    assert oracle.f16c_decode(np.array([code], np.uint16))[0] == np.float32(value)
    assert np.signbit(oracle.f16c_decode(np.array([code], np.uint16))[0]) == np.signbit(value)
    assert oracle.f16c_encode(np.array([value], np.float32))[0] == code


def test_f16c_round_trip_and_rounding():
    codes = np.arange(65536, dtype=np.uint16)
    vals = oracle.f16c_decode(codes)
    # every code is a fixed point of encode(decode(.))
    assert np.array_equal(oracle.f16c_encode(vals), codes)
    # decode is monotone on non-negative codes
    pos = vals[:0x8000]
    assert np.all(np.diff(pos.astype(np.float64)) > 0)
    # saturation above the largest code, round half up between neighbours
    assert oracle.f16c_encode(np.array([3.0, 1e30], np.float32)).tolist() == [0x7FFF, 0x7FFF]
    mid = np.float32((1.0 + (1.0 + 2.0 ** -11)) / 2)
    assert oracle.f16c_encode(np.array([mid], np.float32))[0] == 0x7801


# ---- lattices and layout ----------------------------------------------------------------
@pytest.mark.parametrize("lid,pylat", [(0, get_D2Q9), (1, get_D3Q19), (2, get_D3Q27)])
def test_lattice_tables(lid, pylat):
    c, w, o = oracle.lattice(lid)
    L = pylat()
    assert np.array_equal(c[:, : L.D], L.directions)
    np.testing.assert_allclose(w, L.weights, rtol=0, atol=0)
    assert np.array_equal(o, L.opposite_indices)
    assert abs(w.sum() - 1.0) < 1e-15
    assert L.is_valid_for_esoteric_pull()
    # second moment of the weights is cs^2 (isotropy)
    for a in range(L.D):
        assert abs((w * c[:, a] ** 2).sum() - 1 / 3) < 1e-15


def test_layout_known_answers():
    # 8x8x4 tile on a 16x16x8 grid, Q = 19: offset = lx + 8*(ly + 8*(lz + 4*(q + 19*tile)))
    g = make_grid("D3Q19", (16, 16, 8), (8, 8, 4))
    assert oracle.layout_offset(g, 0, 0, 0, 0, 19) == 0
    assert oracle.layout_offset(g, 1, 0, 0, 0, 19) == 1
    assert oracle.layout_offset(g, 0, 1, 0, 0, 19) == 8
    assert oracle.layout_offset(g, 0, 0, 1, 0, 19) == 64
    assert oracle.layout_offset(g, 0, 0, 0, 1, 19) == 256
    assert oracle.layout_offset(g, 8, 0, 0, 0, 19) == 256 * 19
    assert oracle.layout_offset(g, 0, 8, 0, 0, 19) == 2 * 256 * 19
    assert oracle.layout_offset(g, 0, 0, 4, 0, 19) == 4 * 256 * 19
    assert oracle.layout_offset(g, 15, 15, 7, 18, 19) == 7 + 8 * (7 + 8 * (3 + 4 * (18 + 19 * 7)))
    # the same formula in the package, and a bijection
    lay = g.layouts
    x, y, z, q = np.meshgrid(*(np.arange(n) for n in (16, 16, 8, 19)), indexing="ij")
    off = lay.f_offset(x, y, z, q).ravel()
    assert np.array_equal(np.sort(off), np.arange(off.size))
    assert lay.f_offset(15, 15, 7, 18) == oracle.layout_offset(g, 15, 15, 7, 18, 19)
    # untiled = column-major with q slowest (layoutstruct.mojo:67-69)
    u = make_grid("D2Q9", (6, 5, 1))
    assert oracle.layout_offset(u, 2, 3, 0, 4, 9) == 2 + 6 * 3 + 30 * 4


# ---- invariants of the step ----------------------------------------------------------------
CFGS = [dict(collision_op=c, LES=les, DDF_shift=ddf, use_float16c=f16)
        for c in ("SRT", "TRT", "KBC", "RLBM") for les in (False, True) for ddf, f16 in ((False, False), (True, False),
                                                                                        (True, True))]


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
@pytest.mark.parametrize("meth", [LBM_method.DOUBLE_BUFFER, LBM_method.ESOTERIC_PULL])
@pytest.mark.parametrize("kw", CFGS, ids=[f"{k['collision_op']}-les{k['LES']}-ddf{k['DDF_shift']}-f16{k['use_float16c']}"
                                          for k in CFGS])
def test_rest_state_is_fixed_point(lat, meth, kw):
    shape = {"D2Q9": (8, 6, 1), "D3Q19": (6, 4, 4), "D3Q27": (4, 4, 4)}[lat]
    g = make_grid(lat, shape)
    cfg = LBM_Config(meth, **kw)
    f = initial_f(g, cfg, None)
    flags = np.zeros(g.num_points, np.uint8)
    bc = np.zeros(g.num_points * (g.D + 1), np.float32)
    f2 = f.copy()
    oracle.step(cfg, g, 32, f2 if meth == LBM_method.DOUBLE_BUFFER else f, f, bc, flags, 0.8, True)
    out = f2 if meth == LBM_method.DOUBLE_BUFFER else f
    r = initial_f(g, cfg, None)
    if cfg.use_float16c:
        assert np.abs(out.astype(np.int32) - r.astype(np.int32)).max() <= 1
    else:
        np.testing.assert_allclose(out, r, atol=2e-7)


@pytest.mark.parametrize("lat", ["D2Q9", "D3Q19", "D3Q27"])
@pytest.mark.parametrize("coll", ["SRT", "TRT", "KBC", "RLBM"])
def test_closed_box_conserves_mass_fp64(lat, coll):
    shape = {"D2Q9": (16, 12, 1), "D3Q19": (8, 8, 6), "D3Q27": (6, 6, 6)}[lat]
    g = make_grid(lat, shape, (4, 4, 1) if lat == "D2Q9" else (2, 2, 3))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, collision_op=coll, include_moving_boundary=False)
    flags, bc = ldc_flags(g, cfg, 0.0)
    f = initial_f(g, cfg, np.random.default_rng(1), prec=64, amp=0.03)
    fluid = (g.layouts.from_layout(flags, 1)[..., 0] & 0x0F) != Flags.SOLID
    m0 = oracle.gather(cfg, g, 64, f).sum(0)[fluid].sum()
    f2 = f.copy()
    for _ in range(20):
        oracle.step(cfg, g, 64, f2, f, bc.astype(np.float64), flags, 0.6 if coll == "KBC" else 0.8)
        f, f2 = f2, f
    m1 = oracle.gather(cfg, g, 64, f).sum(0)[fluid].sum()
    assert abs(m1 - m0) < 1e-11 * m0


def test_esoteric_whole_array_conserved_and_matches_double_buffer_periodic():
    g = make_grid("D3Q19", (8, 6, 6), (4, 3, 3))
    rng = np.random.default_rng(3)
    u = rng.uniform(-0.04, 0.04, (3,) + g.shape)
    db, es = LBM_Config(LBM_method.DOUBLE_BUFFER, LES=True), LBM_Config(LBM_method.ESOTERIC_PULL, LES=True)
    fd = np.zeros(g.num_points * 19, np.float64)
    fe = np.zeros_like(fd)
    oracle.init(db, g, 64, fd, 1.0, 0.7, u)
    oracle.init(es, g, 64, fe, 1.0, 0.7, u)
    flags = np.zeros(g.num_points, np.uint8)
    bc = np.zeros(g.num_points * 4)
    fd2 = fd.copy()
    total0 = fe.sum()
    for k in range(6):
        oracle.step(db, g, 64, fd2, fd, bc, flags, 0.7)
        fd, fd2 = fd2, fd
        oracle.step(es, g, 64, fe, fe, bc, flags, 0.7, k % 2 == 0)
    assert np.array_equal(oracle.gather(db, g, 64, fd), oracle.gather(es, g, 64, fe, after_odd=True))
    assert abs(fe.sum() - total0) < 1e-11 * total0


def test_fp32_tracks_fp64_oracle():
    g = make_grid("D3Q19", (10, 10, 10), (5, 5, 5))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER)
    flags, bc = ldc_flags(g, cfg, 0.1)
    f64 = np.zeros(g.num_points * 19)
    oracle.init(cfg, g, 64, f64)
    f32 = f64.astype(np.float32)
    a64, a32 = f64.copy(), f32.copy()
    for _ in range(50):
        oracle.step(cfg, g, 64, a64, f64, bc.astype(np.float64), flags, 0.77)
        f64, a64 = a64, f64
        oracle.step(cfg, g, 32, a32, f32, bc, flags, 0.77)
        f32, a32 = a32, f32
    assert np.abs(f32 - f64).max() < 2e-6


def test_mixed_flags_capture_and_equilibrium_bc():
    """Every branch runs and the captured values equal the oracle's own moments."""
    g = make_grid("D2Q9", (20, 16, 1), (5, 4, 1))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, BCs={Flags.EQUILIBRIUM}, capture_density=True, capture_velocity=True)
    flags, bc = mixed_flags(g, np.random.default_rng(6))
    f = initial_f(g, cfg, np.random.default_rng(7))
    f2 = f.copy()
    oracle.step(cfg, g, 32, f2, f, bc, flags, 0.9)
    assert np.isfinite(f2).all()
    # a cell flagged EQUILIBRIUM with fixed rho, u leaves as f_eq relaxed toward itself (= f_eq)
    bcn = g.layouts.from_layout(bc, 3)
    fl = g.layouts.from_layout(flags, 1)[..., 0]
    fix = (fl == Flags.EQUILIBRIUM) & np.isfinite(bcn[..., 0]) & np.isfinite(bcn[..., 2])
    x, y, _ = np.nonzero(fix)
    i = 0
    out = g.layouts.from_layout(f2, 9)[x[i], y[i], 0]
    ref = np.zeros(g.num_points * 9, np.float32)
    uu = np.zeros((2,) + g.shape)
    uu[:, x[i], y[i], 0] = bcn[x[i], y[i], 0, :2]
    oracle.init(cfg, g, 32, ref, float(bcn[x[i], y[i], 0, 2]), 1.0, uu)
    # init uses one rho for all cells; compare the equilibrium at this cell only
    np.testing.assert_allclose(out, g.layouts.from_layout(ref, 9)[x[i], y[i], 0], atol=2e-7)


# ---- the reference's fixture: Ghia et al. cavity centre lines at Re = 100 ---------------------
def test_ldc_re100_against_ghia_fixture():
    """D2Q9 SRT cavity, lid u = 0.1, tau from Re = 100 with L = N - 1 (units.mojo:123-126,
    examples/LDC.mojo:64-71); centre-line profiles against the Re = 100 columns of
    benchmarks/LDC/ (tests/golden/ghia_re100.json).  Mid-grid bounce-back puts the walls
    half-way between the solid and the first fluid node."""
    N = 96
    U = 0.1
    g = make_grid("D2Q9", (N, N, 1), (16, 16, 1))
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER)
    flags, bc = ldc_flags(g, cfg, U)
    tau = 3 * U * (N - 1) / 100 + 0.5
    f = np.zeros(g.num_points * 9, np.float32)
    oracle.init(cfg, g, 32, f)
    f2 = f.copy()
    for _ in range(12000):
        oracle.step(cfg, g, 32, f2, f, bc, flags, tau)
        f, f2 = f2, f
    _, u = oracle.rho_u(cfg, g, 32, f, bc, flags)
    fix = json.loads((GOLDEN / "ghia_re100.json").read_text())
    # wall-to-wall coordinate s in [0,1] <-> lattice 0.5 + s (N - 2)
    coord = lambda s: 0.5 + np.asarray(s) * (N - 2)  # noqa: E731
    xc = coord(0.5)
    i0 = int(np.floor(xc))
    wx = xc - i0
    ucl = (1 - wx) * u[0, i0, :, 0] + wx * u[0, i0 + 1, :, 0]   # u along the vertical centre line
    vcl = (1 - wx) * u[1, :, i0, 0] + wx * u[1, :, i0 + 1, 0]   # v along the horizontal centre line
    ys, us = np.array(fix["u_vs_y"]).T
    xs, vs = np.array(fix["v_vs_x"]).T
    inner = (ys > 0) & (ys < 1)
    u_sim = np.interp(coord(ys[inner]), np.arange(N), ucl) / U
    v_sim = np.interp(coord(xs[inner]), np.arange(N), vcl) / U
    assert np.abs(u_sim - us[inner]).max() < 0.03, np.c_[ys[inner], u_sim, us[inner]]
    assert np.abs(v_sim - vs[inner]).max() < 0.03, np.c_[xs[inner], v_sim, vs[inner]]


# ---- the reference's DFG cylinder record (tests/golden/dfg_re20.json) --------------------------
def test_dfg_fixture():
    """The fixture holds the DFG targets and the reference's recorded drag for the resolutions the
    GPU test runs (test_fixture_reextracts_from_reference re-extracts it where REF is set)."""
    fix = json.loads((GOLDEN / "dfg_re20.json").read_text())
    assert abs(fix["Cd"] - 5.58) < 0.01 and 0.0 < fix["Cl"] < 0.02
    grids = {tuple(r["grid"]) for r in fix["reference_runs"]}
    assert {(1024, 256), (2560, 512)} <= grids
    for r in fix["reference_runs"]:
        assert abs(r["drag"] - fix["Cd"]) / fix["Cd"] < 0.02


# ---- the oracle's own goldens (tests/golden/oracle_goldens.json) --------------------------------
def test_oracle_goldens():
    """The float32 oracle reproduces the committed SHA-256 digests of its output (f after 6 steps and
    the bc array) on the 192 seeded step cases; the digests of the inputs are checked first, so a
    change of the case recipe (or of numpy's generator) is told apart from a change of the oracle."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_oracle_goldens", GOLDEN / "make_oracle_goldens.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    fix = json.loads((GOLDEN / "oracle_goldens.json").read_text())
    assert fix["steps"] == mod.STEPS and len(fix["cases"]) == len(mod.CASES) == 192
    changed_in, changed_out = [], []
    for c in mod.CASES:
        d_in, d_out = mod.run_case(c)
        want = fix["cases"][mod.case_id(c)]
        if d_in != want["inputs"]:
            changed_in.append(mod.case_id(c))
        elif d_out != want["outputs"]:
            changed_out.append(mod.case_id(c))
    assert not changed_in, f"inputs of {len(changed_in)} cases differ from the fixture's: {changed_in[:4]}"
    assert not changed_out, f"oracle output of {len(changed_out)} cases changed: {changed_out[:4]}"


# ---- the reference's velocity sets (tests/golden/lattices.json) ---------------------------------
@pytest.mark.parametrize("lid,name,pylat", [(0, "D2Q9", get_D2Q9), (1, "D3Q19", get_D3Q19), (2, "D3Q27", get_D3Q27)])
def test_lattices_match_reference_fixture(lid, name, pylat):
    """The oracle's and the package's velocity sets are the reference's: the directions in its order,
    the weights equal to its fractions as float32 (the reference's float_dtype) and the order of the
    stress components (test_fixture_reextracts_from_reference re-extracts it where REF is set)."""
    fix = json.loads((GOLDEN / "lattices.json").read_text())
    ref = fix[name]
    c, w, o = oracle.lattice(lid)
    L = pylat()
    dirs = np.array(ref["directions"])
    assert dirs.shape == (L.Q, L.D)
    assert np.array_equal(c[:, : L.D], dirs) and np.array_equal(L.directions, dirs)
    wref = np.array([a / b for a, b in ref["weights"]], np.float64).astype(np.float32)
    assert np.array_equal(w.astype(np.float32), wref) and np.array_equal(L.weights.astype(np.float32), wref)
    assert all(np.array_equal(dirs[q], -dirs[q + 1]) and o[q] == q + 1 for q in range(1, L.Q, 2))
    assert [list(p) for p in L.stress_indices] == oracle.stress_pairs(L.D) == fix["stress_pairs"][str(L.D)]


@needs_reference
@pytest.mark.parametrize("name,script", [("dfg_re20.json", "make_dfg_fixture.py"),
                                         ("lattices.json", "make_lattice_fixture.py")])
def test_fixture_reextracts_from_reference(name, script):
    """Extracting the fixture again from the reference at REF gives the committed file."""
    import importlib.util
    fix = json.loads((GOLDEN / name).read_text())
    spec = importlib.util.spec_from_file_location(script[:-3], GOLDEN / script)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    assert mod.extract((reference_root() / fix["source"]).read_text()) == fix
