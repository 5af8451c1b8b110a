"""The Mojo binding (mojo_lbm_gb300/mojo/gb300.mojo) agrees with the C header it binds.

No Mojo toolchain exists where this library is built and tested, so the binding is checked as
text: its lbm_config_t / lbm_grid_t structs have the header's fields in order with the matching
Mojo types, and every function it looks up with get_function has the header's parameter and
return types under the C-to-Mojo mapping of the binding (int32_t -> Int32, int64_t -> Int64,
float -> Float32, struct pointers -> UnsafePointer[struct], double[] -> UnsafePointer[Float64],
const char* -> UnsafePointer[UInt8], every other pointer and the handle -> VoidPtr).
"""
from __future__ import annotations

import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "lbm_gb300.h"
BINDING = ROOT / "mojo_lbm_gb300" / "mojo" / "gb300.mojo"

SCALARS = {"int32_t": "Int32", "int64_t": "Int64", "float": "Float32", "uint8_t": "UInt8", "uint32_t": "UInt32", "lbm_status": "Int32"}


def _strip_c_comments(s: str) -> str:
    s = re.sub(r"/\*.*?\*/", " ", s, flags=re.S)
    return re.sub(r"//[^\n]*", " ", s)


def c_struct_fields(name: str) -> list[tuple[str, str]]:
    src = _strip_c_comments(HEADER.read_text())
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", src, re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        out += [(n.strip(), SCALARS[ctype]) for n in names.split(",")]
    return out


def mojo_struct_fields(name: str) -> list[tuple[str, str]]:
    src = BINDING.read_text()
    body = re.search(r"struct " + name + r":\n(.*?)(?:\n\n|\Z)", src, re.S).group(1)
    return re.findall(r"^\s+var (\w+): (\w+)", body, re.M)


def c_to_mojo(ctype: str) -> str:
    t = ctype.replace("const", "").replace(" ", "")
    if t.endswith("**"):
        assert t in ("lbm_handle**", "lbm_batch**"), t
        return "UnsafePointer[VoidPtr]"
    if t.endswith("*"):
        base = t[:-1]
        if base in ("lbm_config_t", "lbm_grid_t"):
            return f"UnsafePointer[{base}]"
        if base == "double":
            return "UnsafePointer[Float64]"
        if base == "char":
            return "UnsafePointer[UInt8]"
        return "VoidPtr"
    return SCALARS[t]


def c_prototypes() -> dict[str, tuple[str, list[str]]]:
    src = _strip_c_comments(HEADER.read_text())
    protos = {}
    for m in re.finditer(r"\b((?:const\s+)?[\w]+\s*\**)\s*\b(lbm_\w+)\s*\(([^;{]*?)\)\s*;", src, re.S):
        ret, name, params = m.group(1), m.group(2), m.group(3).strip()
        types = []
        if params and params != "void":
            for p in params.split(","):
                p = " ".join(p.split())
                arr = re.search(r"\[\d*\]$", p)
                if arr:  # double out[4] -> double*
                    p = p[: arr.start()]
                    ctype = p.rsplit(" ", 1)[0] + "*"
                else:
                    ctype = re.sub(r"\b\w+$", "", p).strip()
                types.append(c_to_mojo(ctype))
        protos[name] = (c_to_mojo(ret), types)
    return protos


def mojo_lookups() -> list[tuple[str, str, list[str]]]:
    src = BINDING.read_text()
    out = []
    for m in re.finditer(r"get_function\[\s*fn \((.*?)\) -> ([\w\[\]]+)\s*\]\(\"(\w+)\"\)", src, re.S):
        args = [a.strip() for a in m.group(1).split(",") if a.strip()]
        out.append((m.group(3), m.group(2), args))
    return out


def test_structs_match_header():
    for name in ("lbm_config_t", "lbm_grid_t"):
        assert mojo_struct_fields(name) == c_struct_fields(name), name


def test_every_lookup_matches_its_prototype():
    protos = c_prototypes()
    lookups = mojo_lookups()
    assert len(lookups) >= 14
    for name, ret, args in lookups:
        assert name in protos, f"{name} is not declared in the header"
        want_ret, want_args = protos[name]
        assert ret == want_ret, (name, ret, want_ret)
        assert args == want_args, (name, args, want_args)


def test_binding_covers_the_step_entry_points():
    names = {n for n, _, _ in mojo_lookups()}
    for must in ("lbm_create", "lbm_destroy", "lbm_double_buffer_step", "lbm_esoteric_pull_step", "lbm_run",
                 "lbm_init_equilibrium", "lbm_compute_rho_u", "lbm_reduce_mass_momentum", "lbm_last_error",
                 "lbm_config_default", "lbm_validate"):
        assert must in names, must
