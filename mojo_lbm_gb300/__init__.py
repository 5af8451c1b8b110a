"""mojo_lbm_gb300: the fused lattice-Boltzmann stream–collide step of JohnCSu/mojo_lbm on GB300.

The compute path is liblbm_gb300.so (hand-written sm_103a CUDA kernels behind the C ABI of
include/lbm_gb300.h).  This package mirrors the reference's host surface — LBM_Config,
LBM_Grid, lattices, UnitSystem, Solver, Assembly, wall set-up and rigid-sphere links — and
drives the library through ctypes with torch CUDA tensors as device buffers.
"""
from ._capi import LBMError, lib
from .config import DoubleBufferConfig, EsotericPullConfig, LBM_Config
from .constants import (DOUBLE_BUFFER, ESOTERIC_PULL, FLUID_NODE, SOLID_NODE, Bounceback_method, Collisions, Flags,
                        LBM_method, cs, cs_squared)
from .grid import LBM_Grid, TiledLayouts
from .lattice import Lattice, get_D2Q9, get_D3Q19, get_D3Q27
from .units import UnitSystem, tau_from_Re

__all__ = [
    "LBMError", "lib", "LBM_Config", "DoubleBufferConfig", "EsotericPullConfig", "DOUBLE_BUFFER", "ESOTERIC_PULL",
    "FLUID_NODE", "SOLID_NODE", "Bounceback_method", "Collisions", "Flags", "LBM_method", "cs", "cs_squared",
    "LBM_Grid", "TiledLayouts", "Lattice", "get_D2Q9", "get_D3Q19", "get_D3Q27", "UnitSystem", "tau_from_Re",
    "Solver", "Assembly",
]


def __getattr__(name):
    # Solver and Assembly pull in the CUDA library / torch lazily
    if name == "Solver":
        from .solver import Solver
        return Solver
    if name == "Assembly":
        from .assembly import Assembly
        return Assembly
    raise AttributeError(name)
