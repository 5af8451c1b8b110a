"""Assembly: owner of the device buffers of one domain (mirrors src/lbm/assembly.mojo:43-269).

f (and f2 for the double buffer), bc and flags live in HBM as torch tensors in the grid's
tiled layout.  flags and bc are painted on the host (numpy) and uploaded by ``upload``;
the initial populations are written on the device by the library's init kernel.
"""
from __future__ import annotations

import numpy as np
import torch

from . import preprocess
from .constants import LBM_method


class Assembly:
    def __init__(self, grid, config, unitSystem=None, device: str | torch.device = "cuda"):
        self.grid = grid
        self.config = config
        self.unitSystem = unitSystem
        self.device = torch.device(device)
        N = grid.num_points
        f_dtype = torch.int16 if config.use_float16c else torch.float32  # uint16 codes stored as int16 bits
        self.f = torch.zeros(N * grid.Q, dtype=f_dtype, device=self.device)
        self.f2 = None if config.lbm_method == LBM_method.ESOTERIC_PULL else torch.zeros_like(self.f)
        self.bc = torch.zeros(N * (grid.D + 1), dtype=torch.float32, device=self.device)
        self.flags = torch.zeros(N, dtype=torch.uint8, device=self.device)
        self.flags_host = np.zeros(N, dtype=np.uint8)
        self.bc_host = np.zeros(N * (grid.D + 1), dtype=np.float32)

    # -- buffer views (assembly.mojo:100-189) ---------------------------------------------
    def get_gpu_tensors_for_double_buffer(self):
        if self.config.lbm_method != LBM_method.DOUBLE_BUFFER:
            raise RuntimeError("This function is only valid if the lbm method is Double Buffer")
        return self.f, self.f2, self.bc, self.flags

    def get_gpu_tensors_for_esoteric_pull(self):
        if self.config.lbm_method != LBM_method.ESOTERIC_PULL:
            raise RuntimeError("This function is only valid if the lbm method is Esoteric Pull")
        return self.f, self.bc, self.flags

    # -- set-up ---------------------------------------------------------------------------
    def set_exterior_walls(self, side: str, boundary_type: int, u=(), rho: float = float("nan"), *,
                           in_lattice_units: bool = True, u_func=None) -> None:
        """Paints one wall into the host flags/bc (assembly.mojo:226-267); call upload() after."""
        units = None if in_lattice_units else self.unitSystem
        if u_func is not None:
            preprocess.set_exterior_walls_with_func(self.grid, self.config, self.flags_host, self.bc_host, side,
                                                    boundary_type, u_func, units, rho)
        else:
            preprocess.set_exterior_walls(self.grid, self.config, self.flags_host, self.bc_host, side,
                                          boundary_type, u, rho, units)

    def upload(self) -> None:
        """Copies the host flags and bc to the device."""
        self.flags.copy_(torch.from_numpy(self.flags_host))
        self.bc.copy_(torch.from_numpy(self.bc_host))

    def initialize_f(self, solver, rho: float = 1.0, tau: float = 1.0, u=None, grad=None) -> None:
        """initialize_f / initialize_fluid_at_rest (assembly.mojo:192-224) on the device.
        u: [D, nx, ny, nz] lattice-unit velocity (None = at rest); grad: [D, D, nx, ny, nz]."""
        ut = None if u is None else torch.as_tensor(np.asarray(u, dtype=np.float32), device=self.device).contiguous()
        gt = None if grad is None else torch.as_tensor(np.asarray(grad, dtype=np.float32),
                                                       device=self.device).contiguous()
        solver.init_equilibrium(self.f, rho, tau, ut, gt)
        if self.f2 is not None:
            self.f2.copy_(self.f)
        torch.cuda.synchronize(self.device)

    def initialize_f_at_rest(self, solver) -> None:
        self.initialize_f(solver, 1.0, 1.0)
