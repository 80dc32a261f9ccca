"""Uniform neighbour grid over the gas particles, rebuilt on the device
(host side of gb_grid_*).

Mirrors core/solvers/neighbor_grid.py:35-136 of the reference: the same
class name, constructor, ``rebuild(pos, h, is_star) -> ngas`` and
``rebuild_all(pos, h) -> ngas``, and the same attributes read by the SPH
kernels (``gsort``, ``cell_start``, ``nx, ny, nz``, ``lo``, ``inv_cell``,
``ngas``, ``max_cells``).  ``gsort`` and ``cell_start`` are int32 device
tensors with the reference's sizes and contents; positions come as the
(n, 4) float32 ``xm`` tensor, smoothing lengths as float32 and ``is_star``
as int32 device tensors.  ``rebuild`` returns the gas count, which waits
for the stream as the reference's host rebuild does; ``rebuild_async``
does not wait.
"""
from __future__ import annotations

import ctypes

import torch

from .. import _lib
from .._dev import ptr, require_cuda, stream_handle


class NeighborGrid:
    def __init__(self, n: int, min_radius: float = 0.0, device=None):
        self.device = require_cuda(device)
        self.n = int(n)
        self.min_radius = float(min_radius)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("gb_grid_create", ctypes.byref(h), self.n, self.min_radius)
        self._h = h
        self.max_cells = int(_lib.load().gb_grid_max_cells(h))
        self.gsort = torch.zeros(max(self.n, 1), dtype=torch.int32, device=self.device)
        self.cell_start = torch.zeros(self.max_cells + 1, dtype=torch.int32, device=self.device)
        self.nx = self.ny = self.nz = 1
        self.lo = (0.0, 0.0, 0.0)
        self.inv_cell = 1.0
        self.ngas = 0

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().gb_grid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _check(self, xm, h, is_star):
        if xm.shape[0] != self.n or h.shape[0] != self.n:
            raise ValueError(f"NeighborGrid was sized for n={self.n}")
        if h.dtype != torch.float32 or not h.is_contiguous():
            raise ValueError("h must be a contiguous float32 tensor")
        if is_star is not None and (is_star.dtype != torch.int32 or not is_star.is_contiguous()
                                    or is_star.shape[0] != self.n):
            raise ValueError("is_star must be a contiguous int32 tensor of length n")

    def _rebuild(self, xm, h, is_star, info):
        self._check(xm, h, is_star)
        _lib.call("gb_grid_rebuild", self._h, ptr(xm, "xm"), h.data_ptr(),
                  is_star.data_ptr() if is_star is not None else None,
                  self.gsort.data_ptr(), self.cell_start.data_ptr(),
                  ctypes.byref(info) if info is not None else None, stream_handle(self.device))

    def rebuild(self, xm: torch.Tensor, h: torch.Tensor, is_star: torch.Tensor | None) -> int:
        """Bin the gas particles (is_star == 0); return the gas count
        (core/solvers/neighbor_grid.py:49-98).  is_star=None bins all
        particles (rebuild_all, :100-136)."""
        info = _lib.GridInfo()
        self._rebuild(xm, h, is_star, info)
        self.ngas = int(info.ngas)
        if self.ngas > 0:
            self.nx, self.ny, self.nz = int(info.nx), int(info.ny), int(info.nz)
            self.lo = (float(info.lo[0]), float(info.lo[1]), float(info.lo[2]))
            self.inv_cell = float(info.inv_cell)
        return self.ngas

    def rebuild_all(self, xm: torch.Tensor, h: torch.Tensor) -> int:
        return self.rebuild(xm, h, None)

    def rebuild_async(self, xm: torch.Tensor, h: torch.Tensor, is_star: torch.Tensor | None = None) -> None:
        """The same rebuild without waiting; the host attributes are not
        updated."""
        self._rebuild(xm, h, is_star, None)

    def launch_count(self) -> int:
        return int(_lib.load().gb_grid_launch_count(self._h))
