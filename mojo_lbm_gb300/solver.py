"""Solver: the host wrapper that launches the fused step (mirrors src/lbm/solver.mojo:35-187).

Every call goes through the C ABI of liblbm_gb300.so; device buffers are torch CUDA tensors
(or raw device addresses) laid out as the grid's tiled layouts.
"""
from __future__ import annotations

import ctypes as C

from . import _capi
from ._capi import check, ptr, stream_ptr
from .constants import LBM_method


class Solver:
    """Creates the library handle for (grid, config) and enqueues steps on a CUDA stream."""

    def __init__(self, grid, config, *, block_dim: int | None = None):
        self.grid = grid
        self.config = config
        self.lbm_method = config.lbm_method
        self._lib = _capi.lib()
        self._cfg = config.to_c()
        self._grid = grid.to_c()
        h = C.c_void_p()
        check(self._lib.lbm_create(C.byref(self._cfg), C.byref(self._grid), C.byref(h)))
        self._h = h
        if block_dim is not None:
            self.set_block_threads(block_dim)

    # -- lifetime --------------------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.lbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_block_threads(self, threads: int) -> None:
        check(self._lib.lbm_set_block_threads(self._h, int(threads)))

    def set_kernel_path(self, path: int) -> None:
        """0 automatic, 1 generic kernel, 2 block-per-tile kernel, 3 cell-pair block-per-tile kernel,
        4 staged block-per-tile kernel (3 and 4: double buffer; identical results in the exact
        arithmetic)."""
        check(self._lib.lbm_set_kernel_path(self._h, int(path)))

    @property
    def kernel_path(self) -> int:
        return int(self._lib.lbm_kernel_path(self._h))

    def device_status(self) -> None:
        """Waits for the device; raises on an error a kernel reported on the device (LBM_ETIMEOUT:
        the staged kernel's bounded wait for its bulk copies ran out)."""
        check(self._lib.lbm_device_status(self._h))

    # -- the step (solver.mojo:81-154) ------------------------------------------------------
    def double_buffer_step(self, f_out, f_in, bc, flags, tau: float, stream=None) -> None:
        check(self._lib.lbm_double_buffer_step(self._h, ptr(f_out), ptr(f_in), ptr(bc), ptr(flags), float(tau),
                                               stream_ptr(stream)))

    def esoteric_pull_step(self, f, bc, flags, tau: float, is_even_step: bool, stream=None) -> None:
        check(self._lib.lbm_esoteric_pull_step(self._h, ptr(f), ptr(bc), ptr(flags), float(tau),
                                               int(bool(is_even_step)), stream_ptr(stream)))

    def even_step(self, assembly, tau: float, stream=None) -> None:
        """f -> f2 (double buffer) or the even in-place step (solver.mojo:159-172)."""
        if self.lbm_method == LBM_method.DOUBLE_BUFFER:
            f_in, f_out, bc, flags = assembly.get_gpu_tensors_for_double_buffer()
            self.double_buffer_step(f_out, f_in, bc, flags, tau, stream)
        else:
            f, bc, flags = assembly.get_gpu_tensors_for_esoteric_pull()
            self.esoteric_pull_step(f, bc, flags, tau, True, stream)

    def odd_step(self, assembly, tau: float, stream=None) -> None:
        """f2 -> f (double buffer) or the odd in-place step (solver.mojo:174-187)."""
        if self.lbm_method == LBM_method.DOUBLE_BUFFER:
            f_in, f_out, bc, flags = assembly.get_gpu_tensors_for_double_buffer()
            self.double_buffer_step(f_in, f_out, bc, flags, tau, stream)
        else:
            f, bc, flags = assembly.get_gpu_tensors_for_esoteric_pull()
            self.esoteric_pull_step(f, bc, flags, tau, False, stream)

    def run(self, f_a, f_b, bc, flags, tau: float, n_steps: int, first_step: int = 0, stream=None) -> None:
        """n_steps steps from a cached CUDA graph; step k reads f_a when first_step + k is even."""
        check(self._lib.lbm_run(self._h, ptr(f_a), ptr(f_b), ptr(bc), ptr(flags), float(tau), int(n_steps),
                                int(first_step), stream_ptr(stream)))

    # -- set-up and outputs -----------------------------------------------------------------
    def init_equilibrium(self, f, rho: float = 1.0, tau: float = 1.0, u=None, grad=None, stream=None) -> None:
        """initialize_f_from_func (preprocess/initial_condition.mojo:86-179) on the device."""
        check(self._lib.lbm_init_equilibrium(self._h, ptr(f), float(rho), float(tau), ptr(u), ptr(grad),
                                             stream_ptr(stream)))

    def compute_rho_u(self, rho, u, f, bc, flags, after_odd_step: bool = False, stream=None) -> None:
        check(self._lib.lbm_compute_rho_u(self._h, ptr(rho), ptr(u), ptr(f), ptr(bc), ptr(flags),
                                          int(bool(after_odd_step)), stream_ptr(stream)))

    def q_criterion(self, q, f, bc, flags, u, tau: float, after_odd_step: bool = False, stream=None) -> None:
        """calculate_Q_criterion (output/Q_criterion.mojo:90-216) into q ([nx, ny, nz]); u is the
        [D, nx, ny, nz] velocity of compute_rho_u for the same state."""
        check(self._lib.lbm_q_criterion(self._h, ptr(q), ptr(f), ptr(bc), ptr(flags), ptr(u), float(tau),
                                        int(bool(after_odd_step)), stream_ptr(stream)))

    def mass_momentum(self, f, flags, after_odd_step: bool = False, stream=None) -> tuple[float, ...]:
        out = (C.c_double * 4)()
        check(self._lib.lbm_reduce_mass_momentum(self._h, ptr(f), ptr(flags), int(bool(after_odd_step)), out,
                                                 stream_ptr(stream)))
        return tuple(out)

    def linkwise_bounceback(self, f, link_force, fluid_ids, dirs, dists, method: int, compute_force: bool = True,
                            q_clamp: float = 0.0, stream=None) -> None:
        n = int(fluid_ids.numel()) if hasattr(fluid_ids, "numel") else len(fluid_ids)
        check(self._lib.lbm_linkwise_bounceback(self._h, ptr(f), ptr(link_force), ptr(fluid_ids), ptr(dirs),
                                                ptr(dists), n, int(method), int(bool(compute_force)),
                                                float(q_clamp), stream_ptr(stream)))

    def set_links(self, fluid_ids, dirs, dists, method: int, q_clamp: float = 0.0, link_force=None,
                  stream=None) -> None:
        """Registers links whose interpolated bounce-back every following double-buffer step applies
        inside the step kernel (lbm_set_links; the node-wise form of
        src/lbm/geometry/nodewise_interpolated_BB.mojo:46-185).  fluid_ids = None removes them."""
        n = 0 if fluid_ids is None else (int(fluid_ids.numel()) if hasattr(fluid_ids, "numel") else len(fluid_ids))
        check(self._lib.lbm_set_links(self._h, ptr(fluid_ids), ptr(dirs), ptr(dists), n, int(method),
                                      float(q_clamp), ptr(link_force), stream_ptr(stream)))

    def sum_link_force(self, link_force, n_links: int, stream=None) -> tuple[float, ...]:
        out = (C.c_double * 3)()
        check(self._lib.lbm_sum_link_force(self._h, ptr(link_force), int(n_links), out, stream_ptr(stream)))
        return tuple(out[: self.grid.D])

    def drag_force(self, node_force, f, flags, fluid_ids, stream=None) -> None:
        n = int(fluid_ids.numel())
        check(self._lib.lbm_drag_force(self._h, ptr(node_force), ptr(f), ptr(flags), ptr(fluid_ids), n,
                                       stream_ptr(stream)))
