"""LBM_Config: the switches of one LBM run (mirrors src/lbm/config.mojo:50-190).

The reference makes these compile-time parameters of its Mojo kernel; here they select one of
the CUDA library's template instantiations when a Solver is created.
"""
from __future__ import annotations

import math
import warnings

from . import _capi
from .constants import Collisions, Flags, LBM_method

_FLAG_SET = {Flags.FLUID, Flags.SOLID, Flags.EQUILIBRIUM}
# LBM_ARITH_EXACT / LBM_ARITH_FAST of the C header
ARITHMETIC = {"exact": 0, "fast": 1}


class LBM_Config:
    """Switches of one run.  Defaults are those of LBM_Config.__init__ (config.mojo:85-99).

    ``Cs`` and ``trt_lambda`` are fixed in the reference (0.1 at steps/collide.mojo:200 and
    3/16 at :214); here they are run-time fields with the same defaults.

    ``arithmetic`` has no counterpart in the reference: ``"exact"`` (default) computes every
    float32 operation in the reference's order, bit-identical to the float32 restatement of the
    reference step; ``"fast"`` rearranges the same operators for fused multiply-add and
    approximate reciprocals and is held to a float32 tolerance of the exact step (block-per-tile
    and batched kernels; other grids run the exact arithmetic).
    """

    def __init__(self, lbm_method: int = LBM_method.DOUBLE_BUFFER, *, collision_op: str = "SRT",
                 LES: bool = False, BCs: set[int] | None = None, DDF_shift: bool = False,
                 use_float16c: bool = False, f_dtype: str | None = None,
                 include_moving_boundary: bool = True, capture_density: bool = False,
                 capture_velocity: bool = False, Cs: float = 0.1, trt_lambda: float = 3.0 / 16.0,
                 arithmetic: str = "exact"):
        if lbm_method not in LBM_method.valid_set:
            raise ValueError("lbm_method not valid")
        self.lbm_method = lbm_method
        self.capture_density = bool(capture_density)
        self.capture_velocity = bool(capture_velocity)
        self.collision_op = collision_op
        self.DDF_shift = bool(DDF_shift)
        self.LES = bool(LES)
        self.KBC = False
        self.include_moving_boundary = bool(include_moving_boundary)
        self.second_moment = bool(LES)
        self.use_float16c = bool(use_float16c)
        if self.use_float16c and f_dtype is not None:
            warnings.warn("Float16c set to True and f_dtype was also specified. Float16c overides the given dtype")
        self.f_dtype = "uint16" if use_float16c else f_dtype
        if self.f_dtype not in (None, "float32", "uint16"):
            raise ValueError("f_dtype must be float32 (float32 arithmetic) or uint16 via use_float16c")
        BCs = set(BCs or ())
        if not BCs:
            self.INCLUDED_BCs = {Flags.FLUID, Flags.SOLID}
        else:
            if not BCs.issubset(_FLAG_SET):
                warnings.warn(f"Some Specified BC types are not standard: {BCs - _FLAG_SET}")
            self.INCLUDED_BCs = {Flags.FLUID, Flags.SOLID} | BCs
        self.Cs = float(Cs)
        self.trt_lambda = float(trt_lambda)
        if not self.collision_op_is_valid():
            raise ValueError(f"Invalid Collision Operator specified: {collision_op}")
        if self.LES and math.isnan(self.Cs):
            raise ValueError("Cs is NaN")
        if arithmetic not in ARITHMETIC:
            raise ValueError(f"arithmetic must be one of {sorted(ARITHMETIC)}")
        self.arithmetic = arithmetic

    def implies_f_noneq(self, *, force: bool = False) -> bool:
        return self.LES or self.collision_op in Collisions.that_need_fneq or force

    def implies_get_adjacent_flags(self, *, force: bool = False) -> bool:
        return self.lbm_method == LBM_method.DOUBLE_BUFFER or self.include_moving_boundary or force

    def implies_bc_is_mutable(self) -> bool:
        return self.capture_density or self.capture_velocity

    def set_f_dtype(self, float_dtype_for_math_ops: str = "float32") -> str:
        return self.f_dtype if self.f_dtype is not None else float_dtype_for_math_ops

    def collision_op_is_valid(self) -> bool:
        return self.collision_op in Collisions.valid_set

    def to_c(self) -> _capi.lbm_config_t:
        c = _capi.lbm_config_t()
        c.lbm_method = self.lbm_method
        c.collision_op = Collisions.ids[self.collision_op]
        c.LES = int(self.LES)
        c.DDF_shift = int(self.DDF_shift)
        c.use_float16c = int(self.use_float16c)
        c.include_moving_boundary = int(self.include_moving_boundary)
        c.include_equilibrium_bc = int(Flags.EQUILIBRIUM in self.INCLUDED_BCs)
        c.capture_density = int(self.capture_density)
        c.capture_velocity = int(self.capture_velocity)
        c.Cs = self.Cs
        c.trt_lambda = self.trt_lambda
        c.arithmetic = ARITHMETIC[self.arithmetic]
        return c

    def __repr__(self) -> str:
        m = "DOUBLE_BUFFER" if self.lbm_method == LBM_method.DOUBLE_BUFFER else "ESOTERIC_PULL"
        return (f"LBM_Config({m}, collision_op={self.collision_op!r}, LES={self.LES}, DDF_shift={self.DDF_shift}, "
                f"use_float16c={self.use_float16c}, include_moving_boundary={self.include_moving_boundary}, "
                f"BCs={sorted(self.INCLUDED_BCs)}, arithmetic={self.arithmetic!r})")


def DoubleBufferConfig(**kw) -> LBM_Config:
    """LBM_Config[LBM_method.DOUBLE_BUFFER] (config.mojo:19)."""
    return LBM_Config(LBM_method.DOUBLE_BUFFER, **kw)


def EsotericPullConfig(**kw) -> LBM_Config:
    """LBM_Config[LBM_method.ESOTERIC_PULL] (config.mojo:23)."""
    return LBM_Config(LBM_method.ESOTERIC_PULL, **kw)
