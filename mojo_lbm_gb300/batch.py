"""Batched persistent step of many domains of different size (lbm_batch_* in the C ABI).

The reference's grid sizes are compile-time parameters (src/lbm/grid.mojo:55-66): one kernel
launch steps one domain.  BatchSolver steps many domains of one lattice and config in one
persistent launch, each exactly as Solver would step it.
"""
from __future__ import annotations

import ctypes as C

from . import _capi
from ._capi import check, ptr, stream_ptr


class BatchSolver:
    def __init__(self, grids, config):
        self.grids = list(grids)
        self.config = config
        self._lib = _capi.lib()
        self._cfg = config.to_c()
        arr = (_capi.lbm_grid_t * len(self.grids))(*[g.to_c() for g in self.grids])
        h = C.c_void_p()
        check(self._lib.lbm_batch_create(C.byref(self._cfg), len(self.grids), arr, C.byref(h)))
        self._h = h
        self._keep = []

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.lbm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_cells(self) -> int:
        return int(self._lib.lbm_batch_cells(self._h))

    def set_domain(self, i: int, f_a, f_b, bc, flags, tau: float) -> None:
        check(self._lib.lbm_batch_set_domain(self._h, int(i), ptr(f_a), ptr(f_b), ptr(bc), ptr(flags), float(tau)))

    def set_links(self, domain, fluid_ids, dirs, dists, method: int, q_clamp: float = 0.0, link_force=None) -> None:
        n = int(fluid_ids.numel())
        self._keep = [domain, fluid_ids, dirs, dists, link_force]
        check(self._lib.lbm_batch_set_links(self._h, ptr(domain), ptr(fluid_ids), ptr(dirs), ptr(dists), n,
                                            int(method), float(q_clamp), ptr(link_force)))

    def set_link_mode(self, fused: bool) -> None:
        """True: the links are applied inside the batched step kernel (LBM_LINKS_FUSED, one kernel per
        step); False: by the link-wise kernel after every step (LBM_LINKS_SEPARATE, the default)."""
        check(self._lib.lbm_batch_set_link_mode(self._h, _capi.LBM_LINKS_FUSED if fused else _capi.LBM_LINKS_SEPARATE))

    def run(self, n_steps: int, first_step: int = 0, stream=None) -> None:
        check(self._lib.lbm_batch_run(self._h, int(n_steps), int(first_step), stream_ptr(stream)))
