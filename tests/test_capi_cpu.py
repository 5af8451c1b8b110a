"""CPU checks of the C ABI library and the host mirror: liblbm_gb300.so loads without a GPU,
exports every function include/lbm_gb300.h declares, validates configurations like the
reference's comptime asserts, and the host-side helpers behave.  No compute call is made."""
from __future__ import annotations

import ctypes as C
import math
import re
from pathlib import Path

import numpy as np
import pytest

from mojo_lbm_gb300 import (DoubleBufferConfig, EsotericPullConfig, Flags, LBM_Config, LBM_Grid, LBM_method, _capi,
                            get_D2Q9, get_D3Q19, get_D3Q27, tau_from_Re)
from mojo_lbm_gb300 import preprocess
from mojo_lbm_gb300.geometry import get_q_for_sphere
from tests.conftest import needs_reference, reference_root

HEADER = Path(__file__).resolve().parents[1] / "include" / "lbm_gb300.h"


def declared_functions() -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(lbm_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    lib = _capi.lib()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} not exported"
    # the ctypes table covers the header exactly
    assert sorted(_capi.SIGNATURES) == names


def test_version_and_empty_error():
    lib = _capi.lib()
    assert b"sm_103a" in lib.lbm_version()


def _validate(cfg, grid):
    c, g = cfg.to_c(), grid.to_c()
    return _capi.lib().lbm_validate(C.byref(c), C.byref(g))


def test_config_defaults_match_reference():
    c = _capi.lbm_config_t()
    assert _capi.lib().lbm_config_default(C.byref(c), 0) == 0
    py = DoubleBufferConfig().to_c()
    for f, _ in _capi.lbm_config_t._fields_:
        assert getattr(c, f) == pytest.approx(getattr(py, f)), f
    assert c.include_moving_boundary == 1 and c.collision_op == 0 and abs(c.Cs - 0.1) < 1e-7
    assert _capi.lib().lbm_config_default(C.byref(c), 7) == _capi.LBM_EINVAL


def test_validate_rules():
    lib = _capi.lib()
    ok = LBM_Grid(get_D3Q19(), 16, 16, 16, (8, 8, 4))
    assert _validate(DoubleBufferConfig(), ok) == 0
    for cfg in (EsotericPullConfig(use_float16c=True, DDF_shift=True, LES=True), DoubleBufferConfig(collision_op="KBC")):
        assert _validate(cfg, ok) == 0
    # lattice dimension must match the grid (grid.mojo:345-365)
    g = _capi.lbm_grid_t(0, 16, 16, 4, 16, 16, 4)
    c = DoubleBufferConfig().to_c()
    assert lib.lbm_validate(C.byref(c), C.byref(g)) == _capi.LBM_EINVAL
    assert b"dimension" in lib.lbm_last_error()
    # tile must divide the grid (grid.mojo:301-305)
    g = _capi.lbm_grid_t(1, 16, 16, 16, 6, 8, 4)
    assert lib.lbm_validate(C.byref(c), C.byref(g)) == _capi.LBM_EINVAL
    assert b"divide" in lib.lbm_last_error()
    # invalid collision operator (config.mojo:153)
    c.collision_op = 9
    g = _capi.lbm_grid_t(1, 16, 16, 16, 8, 8, 4)
    assert lib.lbm_validate(C.byref(c), C.byref(g)) == _capi.LBM_EINVAL
    # element counts
    assert lib.lbm_f_elements(C.byref(g)) == 19 * 4096
    assert lib.lbm_bc_elements(C.byref(g)) == 4 * 4096
    assert lib.lbm_flag_elements(C.byref(g)) == 4096
    assert [lib.lbm_lattice_q(i) for i in range(4)] == [9, 19, 27, -1]
    assert [lib.lbm_lattice_d(i) for i in range(4)] == [2, 3, 3, -1]


def test_validate_edges():
    """Smallest and largest grids, extents, and the Smagorinsky constant."""
    lib = _capi.lib()
    c = DoubleBufferConfig().to_c()

    def check(grid, cfg=c):
        return lib.lbm_validate(C.byref(cfg), C.byref(grid))

    # the smallest grids of each dimension (check_model_match_dim counts extents above 1)
    assert check(_capi.lbm_grid_t(0, 2, 2, 1, 1, 1, 1)) == 0
    assert check(_capi.lbm_grid_t(1, 2, 2, 2, 2, 2, 2)) == 0
    assert check(_capi.lbm_grid_t(1, 1, 1, 1, 1, 1, 1)) == _capi.LBM_EINVAL
    assert b"dimension" in lib.lbm_last_error()
    for g in (_capi.lbm_grid_t(1, 0, 16, 16, 8, 8, 4), _capi.lbm_grid_t(1, 16, -16, 16, 8, 8, 4)):
        assert check(g) == _capi.LBM_EINVAL and b"positive" in lib.lbm_last_error()
    assert check(_capi.lbm_grid_t(1, 16, 16, 16, 0, 8, 4)) == _capi.LBM_EINVAL
    assert b"tile extents" in lib.lbm_last_error()
    # cell indices are 32-bit: 2^32 cells are refused, one row fewer is accepted
    assert check(_capi.lbm_grid_t(0, 65536, 65536, 1, 16, 16, 1)) == _capi.LBM_EINVAL
    assert b"2^32" in lib.lbm_last_error()
    assert check(_capi.lbm_grid_t(0, 65536, 65520, 1, 16, 16, 1)) == 0
    # Cs is read only with LES: there a NaN or a negative value is refused, without LES any value
    g = _capi.lbm_grid_t(1, 16, 16, 16, 8, 8, 4)
    for les, cs, ok in ((False, float("nan"), True), (True, float("nan"), False), (True, -0.1, False),
                        (False, -0.1, True), (True, 0.0, True)):
        cc = DoubleBufferConfig(LES=les).to_c()
        cc.Cs = cs
        assert (check(g, cc) == 0) == ok, (les, cs)
    # arithmetic: LBM_ARITH_EXACT (0) or LBM_ARITH_FAST (1)
    for ar, ok in ((0, True), (1, True), (2, False), (-1, False)):
        cc = DoubleBufferConfig().to_c()
        cc.arithmetic = ar
        assert (check(g, cc) == 0) == ok, ar
    assert DoubleBufferConfig(arithmetic="fast").to_c().arithmetic == 1
    with pytest.raises(ValueError):
        DoubleBufferConfig(arithmetic="approximate")


def test_handle_calls_reject_null():
    lib = _capi.lib()
    assert lib.lbm_double_buffer_step(None, None, None, None, None, 0.8, None) == _capi.LBM_EINVAL
    assert lib.lbm_destroy(None) == 0
    assert lib.lbm_float16c_encode(None, None, 0, None) == 0       # empty is a no-op
    assert lib.lbm_float16c_encode(None, None, 5, None) == _capi.LBM_EINVAL


def test_python_config_mirror():
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, LES=True, BCs={Flags.EQUILIBRIUM})
    assert cfg.implies_f_noneq() and cfg.second_moment
    assert cfg.INCLUDED_BCs == {0, 1, 2}
    assert cfg.to_c().include_equilibrium_bc == 1
    assert not EsotericPullConfig(include_moving_boundary=False).implies_get_adjacent_flags()
    assert DoubleBufferConfig(include_moving_boundary=False).implies_get_adjacent_flags()
    assert EsotericPullConfig(use_float16c=True).set_f_dtype("float32") == "uint16"
    assert LBM_Config(collision_op="KBC").implies_f_noneq()
    with pytest.raises(ValueError):
        LBM_Config(collision_op="MRT")
    with pytest.warns(UserWarning):
        LBM_Config(use_float16c=True, f_dtype="float32")


def test_grid_rules_and_units():
    with pytest.raises(ValueError):
        LBM_Grid(get_D2Q9(), 16, 16, 4)
    with pytest.raises(ValueError):
        LBM_Grid(get_D3Q27(), 16, 16, 16, (5, 8, 8))
    g = LBM_Grid(get_D2Q9(), 32, 16, 1, 8)
    assert g.tile_shape == (8, 8, 1)
    assert LBM_Grid(get_D3Q19(), 16, 16, 16, 4).tile_shape == (4, 4, 4)
    assert LBM_Grid(get_D3Q19(), 16, 8, 8).tile_shape == (16, 8, 8)
    # tau from Re (units.mojo:123-126): the benchmark's 256^3 case, u = 0.1, Re = 100
    assert tau_from_Re(0.1, 255, 100) == pytest.approx(1.265)
    gg = LBM_Grid(get_D3Q19(), 256, 256, 256, 8, dx=1.0 / 255)
    units = gg.get_UnitSystem_with_Re(1.0, 0.1, 1.0, Re=100.0)
    assert units.tau == pytest.approx(1.265)
    # benchmarks/D3.mojo:39-46: U = 0.05, Re = 100, L = 256
    assert tau_from_Re(0.05, 256, 100) == pytest.approx(0.884)


def test_exterior_walls_and_errors():
    g = LBM_Grid(get_D3Q19(), 8, 8, 8, (4, 4, 4))
    cfg = DoubleBufferConfig()
    flags = np.zeros(g.num_points, np.uint8)
    bc = np.zeros(g.num_points * 4, np.float32)
    preprocess.set_exterior_walls(g, cfg, flags, bc, "+Y", Flags.SOLID, [0.1, 0, 0], 1.0)
    nat = g.layouts.from_layout(flags, 1)[..., 0]
    assert (nat[:, 7, :] == Flags.SOLID).all() and nat[:, :7, :].max() == 0
    b = g.layouts.from_layout(bc, 4)
    assert np.allclose(b[:, 7, :, 0], 0.1) and np.allclose(b[:, 7, :, 3], 1.0)
    with pytest.raises(ValueError, match="Side not valid"):
        preprocess.set_exterior_walls(g, cfg, flags, bc, "+W", Flags.SOLID, [0, 0, 0], 1.0)
    with pytest.raises(ValueError, match="valid boundary types"):
        preprocess.set_exterior_walls(g, cfg, flags, bc, "+X", Flags.EQUILIBRIUM, [], 1.0)
    with pytest.raises(ValueError, match="Solid"):
        preprocess.set_exterior_walls(g, cfg, flags, bc, "+X", Flags.SOLID, [0, 0, 0])
    with pytest.raises(ValueError, match="include_moving_boundary"):
        preprocess.set_exterior_walls(g, DoubleBufferConfig(include_moving_boundary=False), flags, bc, "+X",
                                      Flags.SOLID, [0.1, 0, 0], 1.0)
    eq = DoubleBufferConfig(BCs={Flags.EQUILIBRIUM})
    preprocess.set_exterior_walls(g, eq, flags, bc, "+X", Flags.EQUILIBRIUM, [], 1.0)
    b = g.layouts.from_layout(bc, 4)
    assert np.isnan(b[7, 3, 3, :3]).all() and b[7, 3, 3, 3] == 1.0
    # parabolic inlet through a function (examples/CylinderFlow2D-style)
    g2 = LBM_Grid(get_D2Q9(), 16, 12, 1, (4, 4, 1), dx=1 / 11)
    f2 = np.zeros(g2.num_points, np.uint8)
    b2 = np.zeros(g2.num_points * 3, np.float32)
    preprocess.set_exterior_walls_with_func(g2, cfg, f2, b2, "-X", Flags.SOLID,
                                            lambda x, y, z: (0.05 * 4 * y * (1 - y), 0 * y), None, 1.0)
    prof = g2.layouts.from_layout(b2, 3)[0, :, 0, 0]
    assert prof.max() == pytest.approx(0.05 * 4 * (5 / 11) * (6 / 11), rel=1e-6)


def test_sphere_link_parameter():
    c = np.array([0.0, 0.0, 0.0])
    q = get_q_for_sphere(np.array([2.0, 0, 0]), np.array([1.0, 0, 0]), c, 1.5)
    assert q == pytest.approx(0.5)
    q = get_q_for_sphere(np.array([1.0, 1.0, 0]), np.array([0.0, 0.0, 0]), c, 1.0)
    assert 0 <= q <= 1 and q == pytest.approx(1 - 1 / math.sqrt(2))


def test_flags_and_config_defaults_match_reference_fixture():
    """The node flags (package, C header) and LBM_Config's keyword defaults (package and
    lbm_config_default) are the reference's, as extracted into tests/golden/constants.json."""
    import json
    golden = Path(__file__).with_name("golden")
    fix = json.loads((golden / "constants.json").read_text())
    header = HEADER.read_text()
    assert len(fix["flags"]) == 7
    for name, value in fix["flags"].items():
        assert getattr(Flags, name) == value, name
        m = re.search(rf"LBM_FLAG_{name}\s*=\s*(0x[0-9a-fA-F]+|\d+)", header)
        assert m and int(m.group(1), 0) == value, name
    d = fix["config_defaults"]
    py = LBM_Config()
    c = _capi.lbm_config_t()
    assert _capi.lib().lbm_config_default(C.byref(c), 0) == 0
    for k in ("LES", "DDF_shift", "use_float16c", "include_moving_boundary", "capture_density", "capture_velocity"):
        assert getattr(py, k) == d[k] and bool(getattr(c, k)) == d[k], k
    assert py.collision_op == d["collision_op"] == "SRT" and c.collision_op == 0
    # BCs = {} is the reference's default, to which it always adds FLUID and SOLID
    assert d["BCs"] == [] and py.INCLUDED_BCs == {Flags.FLUID, Flags.SOLID} and c.include_equilibrium_bc == 0
    assert d["f_dtype"] is None and py.f_dtype is None


@needs_reference
def test_constants_fixture_reextracts_from_reference():
    """Extracting the flags and LBM_Config defaults again from the reference at REF gives the
    committed fixture."""
    import importlib.util
    import json
    golden = Path(__file__).with_name("golden")
    fix = json.loads((golden / "constants.json").read_text())
    ref = reference_root()
    spec = importlib.util.spec_from_file_location("make_constants_fixture", golden / "make_constants_fixture.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    assert mod.extract((ref / fix["flags_source"]).read_text(), (ref / fix["config_source"]).read_text()) == fix
