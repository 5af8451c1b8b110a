"""ctypes binding of the C ABI in include/lbm_gb300.h.

The shared library is built in place by ``mojo_lbm_gb300._build``.  Loading it needs no GPU;
every compute entry point needs one.  If the library is missing the import of a compute
function raises, so no CPU path ever stands in for the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "liblbm_gb300.so"

LBM_OK, LBM_EINVAL, LBM_ECUDA, LBM_ENAN, LBM_ETIMEOUT, LBM_ENOMEM, LBM_EUNSUPPORTED = range(7)
LBM_LINKS_SEPARATE, LBM_LINKS_FUSED = 0, 1
STATUS_NAMES = {0: "LBM_OK", 1: "LBM_EINVAL", 2: "LBM_ECUDA", 3: "LBM_ENAN", 4: "LBM_ETIMEOUT",
                5: "LBM_ENOMEM", 6: "LBM_EUNSUPPORTED"}


class LBMError(RuntimeError):
    """A C-ABI call returned a status other than LBM_OK."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class lbm_config_t(C.Structure):
    _fields_ = [("lbm_method", C.c_int32), ("collision_op", C.c_int32), ("LES", C.c_int32),
                ("DDF_shift", C.c_int32), ("use_float16c", C.c_int32),
                ("include_moving_boundary", C.c_int32), ("include_equilibrium_bc", C.c_int32),
                ("capture_density", C.c_int32), ("capture_velocity", C.c_int32),
                ("Cs", C.c_float), ("trt_lambda", C.c_float), ("arithmetic", C.c_int32)]


class lbm_grid_t(C.Structure):
    _fields_ = [("lattice", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("tx", C.c_int32), ("ty", C.c_int32), ("tz", C.c_int32)]


class lbm_closure_t(C.Structure):
    _fields_ = [("w1", C.c_float * 256), ("b1", C.c_float * 32), ("w2", C.c_float * 1024), ("b2", C.c_float * 32),
                ("w3", C.c_float * 32), ("b3", C.c_float), ("nu_scale", C.c_float),
                ("feat_mean", C.c_float * 8), ("feat_scale", C.c_float * 8), ("feat_lo", C.c_float * 8),
                ("feat_hi", C.c_float * 8)]


class lbm_tune_result_t(C.Structure):
    _fields_ = [("tx", C.c_int32), ("ty", C.c_int32), ("tz", C.c_int32), ("lbm_method", C.c_int32),
                ("mlups", C.c_float), ("n_candidates", C.c_int32)]


_vp = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64
_f32 = C.c_float
_CFG = C.POINTER(lbm_config_t)
_GRID = C.POINTER(lbm_grid_t)

# name -> (restype, argtypes); every function declared in include/lbm_gb300.h
SIGNATURES = {
    "lbm_config_default": (_i32, [_CFG, _i32]),
    "lbm_validate": (_i32, [_CFG, _GRID]),
    "lbm_lattice_q": (_i32, [_i32]),
    "lbm_lattice_d": (_i32, [_i32]),
    "lbm_f_elements": (_i64, [_GRID]),
    "lbm_bc_elements": (_i64, [_GRID]),
    "lbm_flag_elements": (_i64, [_GRID]),
    "lbm_create": (_i32, [_CFG, _GRID, C.POINTER(_vp)]),
    "lbm_destroy": (_i32, [_vp]),
    "lbm_set_block_threads": (_i32, [_vp, _i32]),
    "lbm_set_kernel_path": (_i32, [_vp, _i32]),
    "lbm_kernel_path": (_i32, [_vp]),
    "lbm_device_status": (_i32, [_vp]),
    "lbm_debug_stage_extra_bytes": (_i32, [_vp, C.c_uint32]),
    "lbm_stage_segments": (_i32, [_i32, _i32, _i32, _i32, _i32, _vp, _i32, _vp]),
    "lbm_double_buffer_step": (_i32, [_vp, _vp, _vp, _vp, _vp, _f32, _vp]),
    "lbm_esoteric_pull_step": (_i32, [_vp, _vp, _vp, _vp, _f32, _i32, _vp]),
    "lbm_run": (_i32, [_vp, _vp, _vp, _vp, _vp, _f32, _i64, _i64, _vp]),
    "lbm_init_equilibrium": (_i32, [_vp, _vp, _f32, _f32, _vp, _vp, _vp]),
    "lbm_compute_rho_u": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i32, _vp]),
    "lbm_q_criterion": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _f32, _i32, _vp]),
    "lbm_reduce_mass_momentum": (_i32, [_vp, _vp, _vp, _i32, C.POINTER(C.c_double), _vp]),
    "lbm_reduce_mass_momentum_noalloc": (_i32, [_CFG, _GRID, _vp, _vp, _i32, C.POINTER(C.c_double), _vp]),
    "lbm_linkwise_bounceback": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _i32, _i32, _f32, _vp]),
    "lbm_set_links": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _f32, _vp, _vp]),
    "lbm_sum_link_force": (_i32, [_vp, _vp, _i64, C.POINTER(C.c_double), _vp]),
    "lbm_drag_force": (_i32, [_vp, _vp, _vp, _vp, _vp, _i64, _vp]),
    "lbm_batch_create": (_i32, [_CFG, _i32, _GRID, C.POINTER(_vp)]),
    "lbm_batch_destroy": (_i32, [_vp]),
    "lbm_batch_set_domain": (_i32, [_vp, _i32, _vp, _vp, _vp, _vp, _f32]),
    "lbm_batch_set_links": (_i32, [_vp, _vp, _vp, _vp, _vp, _i64, _i32, _f32, _vp]),
    "lbm_batch_set_link_mode": (_i32, [_vp, _i32]),
    "lbm_batch_run": (_i32, [_vp, _i64, _i64, _vp]),
    "lbm_batch_cells": (_i64, [_vp]),
    "lbm_set_closure": (_i32, [_vp, C.POINTER(lbm_closure_t)]),
    "lbm_mlp_forward": (_i32, [_vp, _vp, _i64, _f32, _vp, _vp]),
    "lbm_mlp_backward": (_i32, [_vp, _vp, _vp, _i64, _f32, _vp, _vp]),
    "lbm_mlp_adam": (_i32, [_vp, _vp, _vp, _vp, _i32, _f32, _f32, _f32, _f32, _i32, _vp]),
    "lbm_tune_candidates": (_i32, [_i32, _i32, _i32, _i32, _vp, _i32]),
    "lbm_autotune": (_i32, [_CFG, _i32, _i32, _i32, _i32, _vp, _vp, _i32, _i32, C.POINTER(lbm_tune_result_t),
                            _vp]),
    "lbm_paint_wall": (_i32, [_CFG, _GRID, _vp, _vp, _i32, C.c_uint8, C.POINTER(_f32), _f32, _vp]),
    "lbm_paint_wall_values": (_i32, [_CFG, _GRID, _vp, _vp, _i32, C.c_uint8, _vp, _f32, _vp]),
    "lbm_paint_sphere": (_i32, [_GRID, _vp, C.POINTER(_f32), _f32, C.POINTER(_f32), _f32, _vp]),
    "lbm_paint_box": (_i32, [_GRID, _vp, C.POINTER(_f32), C.POINTER(_f32), C.POINTER(_f32), _f32, _vp]),
    "lbm_float16c_encode": (_i32, [_vp, _vp, _i64, _vp]),
    "lbm_float16c_decode": (_i32, [_vp, _vp, _i64, _vp]),
    "lbm_last_error": (C.c_char_p, []),
    "lbm_version": (C.c_char_p, []),
}

_lib = None


def lib() -> C.CDLL:
    """Loads liblbm_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                " (the CUDA library is the only compute path)")
        h = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def check(status: int) -> None:
    """Raises LBMError with the library's message when status is not LBM_OK."""
    if status != LBM_OK:
        raise LBMError(status, lib().lbm_last_error().decode())


def ptr(x) -> int | None:
    """Device (or host) address of a torch tensor, an int, or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def stream_ptr(stream) -> int | None:
    """cudaStream_t of a torch.cuda.Stream (None = the legacy default stream)."""
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream
