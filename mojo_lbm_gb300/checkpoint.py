"""Checkpoint and resume of a run: the lattices (both buffers of the double buffer, or the one
esoteric-pull lattice), flags and boundary values as raw arrays, with a JSON header naming the
configuration, the grid and its tiled layout, the step count and tau.  No counterpart in the
reference (its drivers keep everything in memory).

Resuming is exact: the arrays are written and read back bit for bit, and the header carries the
parity of the next step (which buffer it reads; the esoteric-pull load pattern), so N steps give
the same populations as N/2 steps, a save, a load and N/2 more.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

FORMAT = "mojo_lbm_gb300 checkpoint 1"


def _to_host(a):
    if a is None:
        return None
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy()
    return np.asarray(a)


def _config_fields(config) -> dict:
    return {"lbm_method": int(config.lbm_method), "collision_op": config.collision_op, "LES": bool(config.LES),
            "DDF_shift": bool(config.DDF_shift), "use_float16c": bool(config.use_float16c),
            "include_moving_boundary": bool(config.include_moving_boundary),
            "BCs": sorted(int(b) for b in config.INCLUDED_BCs),
            "capture_density": bool(config.capture_density), "capture_velocity": bool(config.capture_velocity),
            "Cs": float(config.Cs), "trt_lambda": float(config.trt_lambda),
            "arithmetic": getattr(config, "arithmetic", "exact")}


def save(path, grid, config, *, f, bc, flags, step: int, tau: float, f2=None, extra: dict | None = None) -> Path:
    """Writes <path> (an .npz) holding f (and f2 for the double buffer), bc, flags and the header.
    Tensors may live on the GPU; they are copied to the host."""
    path = Path(path)
    header = {
        "format": FORMAT,
        "config": _config_fields(config),
        "grid": {"lattice": int(grid.lattice.id), "shape": list(grid.shape), "tile": list(grid.tile_shape)},
        "step": int(step),
        "tau": float(tau),
        "next_reads": "f" if int(step) % 2 == 0 else "f2",  # double buffer: step k reads f when k is even
        "esoteric_next_even": int(step) % 2 == 0,           # esoteric pull: parity of the next step
        "extra": extra or {},
    }
    arrays = {"f": _to_host(f), "bc": _to_host(bc), "flags": _to_host(flags)}
    if f2 is not None:
        arrays["f2"] = _to_host(f2)
    np.savez(path, header=json.dumps(header), **arrays)
    return path if path.suffix == ".npz" else path.with_suffix(path.suffix + ".npz")


def load(path, grid=None, config=None, device=None) -> dict:
    """Reads a checkpoint; with grid / config given, checks that they match the header (layout,
    lattice and the switches that change the stored bytes).  With device, arrays come back as
    torch tensors on it.  Returns {"header", "f", "f2" (or None), "bc", "flags"}."""
    with np.load(Path(path), allow_pickle=False) as d:
        header = json.loads(str(d["header"]))
        out = {"header": header, "f": d["f"], "f2": d["f2"] if "f2" in d.files else None, "bc": d["bc"],
               "flags": d["flags"]}
    if header.get("format") != FORMAT:
        raise ValueError(f"not a checkpoint of this format: {header.get('format')!r}")
    if grid is not None:
        g = header["grid"]
        if (g["lattice"], tuple(g["shape"]), tuple(g["tile"])) != (grid.lattice.id, tuple(grid.shape),
                                                                    tuple(grid.tile_shape)):
            raise ValueError("checkpoint grid (lattice, shape, tile) differs from the given grid")
    if config is not None:
        c, h = _config_fields(config), header["config"]
        for k in ("lbm_method", "DDF_shift", "use_float16c"):
            if c[k] != h[k]:
                raise ValueError(f"checkpoint {k} = {h[k]} differs from the configuration's {c[k]}")
    if device is not None:
        import torch
        for k in ("f", "f2", "bc", "flags"):
            if out[k] is not None:
                a = out[k]
                out[k] = torch.from_numpy(a.view(np.int16) if a.dtype == np.uint16 else a).to(device)
    return out
