"""Batched direct N^2 integration of many independent systems (host side of
gb_batch_*).  All systems share G, eps and dt; each evolves exactly as a
separate Engine(gravity_mode="direct") would (core/engine.py:108-116).

    b = DirectBatch([pos_vel_mass, ...], G=1.0, softening=0.02)
    b.run(dt, nsteps)              # one persistent launch per step, CUDA graph
    b.run_loop(dt, nsteps)         # per-system loop of the plain kernel

variant=1 runs the symmetric pass (each unordered pair of a system once).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._dev import ptr, require_cuda, stream_handle


def shard_systems(sizes, rank: int, world: int) -> list:
    """Indices of the systems rank `rank` of `world` integrates when a batch
    is split across GPUs: longest-processing-time assignment by N^2 (each
    system whole on one rank, no exchange between ranks), deterministic on
    every rank."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError(f"bad rank {rank} of {world}")
    cost = np.asarray(sizes, dtype=np.float64) ** 2
    order = sorted(range(len(cost)), key=lambda s: (-cost[s], s))
    load = [0.0] * world
    owner = [0] * len(cost)
    for s in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[s] = r
        load[r] += cost[s]
    return [s for s in range(len(cost)) if owner[s] == rank]


class DirectBatch:
    def __init__(self, systems, G: float = 1.0, softening: float = 0.02, device=None,
                 plain_fp32: bool = False, tiles=None, variant: int = 0):
        if not systems:
            raise ValueError("DirectBatch needs at least one system")
        self.device = require_cuda(device)
        self.G = float(G)
        self.eps2 = float(softening) ** 2
        self.plain = bool(plain_fp32)
        self.sizes = np.array([np.asarray(p).reshape(-1, 3).shape[0] for p, _, _ in systems],
                              dtype=np.int64)
        self.offsets = np.concatenate(([0], np.cumsum(self.sizes)))
        n = int(self.offsets[-1])
        xm = np.empty((n, 4), np.float32)
        v4 = np.zeros((n, 4), np.float32)
        for s, (p, v, m) in enumerate(systems):
            o0, o1 = self.offsets[s], self.offsets[s + 1]
            xm[o0:o1, :3] = np.asarray(p).reshape(-1, 3)
            xm[o0:o1, 3] = np.asarray(m).reshape(-1)
            v4[o0:o1, :3] = np.asarray(v).reshape(-1, 3)
        h = ctypes.c_void_p()
        sizes = np.ascontiguousarray(self.sizes)
        with torch.cuda.device(self.device):
            _lib.call("gb_batch_create", ctypes.byref(h), sizes.ctypes.data_as(ctypes.c_void_p),
                      int(sizes.size))
            self._h = h
            self.xm = torch.from_numpy(xm).to(self.device)
            self.v4 = torch.from_numpy(v4).to(self.device)
            self.a4 = torch.zeros_like(self.xm)
            if tiles is not None:
                self.set_tiles(*tiles)
            if variant:
                self.set_variant(variant)
            self.compute_acc()

    @property
    def n_total(self) -> int:
        return int(self.offsets[-1])

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().gb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tiles(self, k: int, warps: int, ctas_per_sm: int = 0):
        _lib.call("gb_batch_set_tiles", self._h, int(k), int(warps), int(ctas_per_sm))

    def set_variant(self, variant: int):
        """Force pass: 0 one pass per target (default), 1 symmetric (each
        unordered pair of a system once; allocates its tile-pair scratch)."""
        _lib.call("gb_batch_set_variant", self._h, int(variant))

    def _flags(self, graph=False):
        return (_lib.GB_PLAIN_FP32 if self.plain else 0) | (_lib.GB_USE_GRAPH if graph else 0)

    def compute_acc(self):
        _lib.call("gb_batch_acc", self._h, ptr(self.xm, "xm"), ptr(self.a4, "acc"), self.G,
                  self.eps2, self._flags(), stream_handle(self.device))

    def run(self, dt: float, nsteps: int, graph: bool = True):
        """nsteps KDK steps of every system: one persistent force launch and
        one fix-up per step; with graph=True the loop replays a CUDA graph."""
        _lib.call("gb_batch_kdk", self._h, ptr(self.xm, "xm"), ptr(self.v4, "vel"),
                  ptr(self.a4, "acc"), self.G, self.eps2, float(dt), int(nsteps),
                  self._flags(graph), stream_handle(self.device))

    def run_loop(self, dt: float, nsteps: int):
        """The same steps through the single-system kernel, system by system."""
        _lib.call("gb_batch_kdk_loop", self._h, ptr(self.xm, "xm"), ptr(self.v4, "vel"),
                  ptr(self.a4, "acc"), self.G, self.eps2, float(dt), int(nsteps),
                  self._flags(), stream_handle(self.device))

    def launch_count(self) -> int:
        return int(_lib.load().gb_batch_launch_count(self._h))

    def interactions_per_step(self) -> int:
        return int((self.sizes.astype(np.float64) ** 2).sum())

    def system(self, s: int):
        """(pos, vel, mass) of system s as float64 numpy arrays."""
        o0, o1 = int(self.offsets[s]), int(self.offsets[s + 1])
        xm = self.xm[o0:o1].double().cpu().numpy()
        v = self.v4[o0:o1].double().cpu().numpy()
        return xm[:, :3], v[:, :3], xm[:, 3]

    def state_arrays(self):
        return (self.xm.detach().clone(), self.v4.detach().clone(), self.a4.detach().clone())

    def restore(self, arrays):
        xm, v4, a4 = arrays
        self.xm.copy_(xm)
        self.v4.copy_(v4)
        self.a4.copy_(a4)
