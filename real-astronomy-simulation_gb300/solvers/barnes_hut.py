"""LBVH Barnes-Hut on the GB300 (host side of gb_bh_*).

Mirrors ``BarnesHut(n, theta, softening, max_stack).compute(pos, mass, acc)``
(core/solvers/barnes_hut.py:220-259).  Every stage (Morton keys, stable
sort, Karras build, node summaries, traversal) runs on the device; keys,
order and topology are bit-identical to the reference's and each particle
accepts the same node set.  Extra keyword arguments: ``key_bits`` (21 = the
reference's 63-bit keys, 10 = 30-bit keys), ``G`` (the reference compiles
core/units.py:21 into its traversal) and ``check``: every call waits for the
device and raises GravityError (GB_ESTACK) when the max_stack rule dropped
work, or (GB_EINVAL) on non-finite positions, where the reference drops
subtrees silently (core/solvers/barnes_hut.py:212).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib, units
from .._dev import empty4, field_values, pick_device, ptr, require_cuda, stream_handle, write_rows

EXPORTS = {"code": (0, np.uint64, 1, 0), "order": (1, np.int32, 1, 0),
           "left": (2, np.int32, 1, -1), "right": (3, np.int32, 1, -1),
           "parent": (4, np.int32, 2, -1), "nmass": (5, np.float64, 2, -1),
           "com": (6, np.float64, 2, -1), "nmin": (7, np.float64, 2, -1),
           "nmax": (8, np.float64, 2, -1)}
_TORCH = {np.uint64: torch.int64, np.int32: torch.int32, np.float64: torch.float64}


class BarnesHut:
    def __init__(self, n: int, theta: float = 0.6, softening: float = 0.1,
                 max_stack: int = 64, *, key_bits: int = 21, G: float = units.G,
                 check: bool = False, device=None):
        self.device = require_cuda(device)
        self.n = int(n)
        self.theta = float(theta)
        self.theta2 = self.theta ** 2
        self.softening = float(softening)
        self.eps2 = self.softening ** 2
        self.max_stack = int(max_stack)
        self.key_bits = int(key_bits)
        self.G = float(G)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("gb_bh_create", ctypes.byref(h), max(self.n, 1), self.key_bits)
        self._h = h
        self._last_n = 0
        self._out3 = None
        self.check = bool(check)
        if self.check:
            _lib.call("gb_bh_set_check", h, 1)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().gb_bh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _n(self, xm) -> int:
        n = xm.shape[0]
        if n > self.n:
            raise ValueError(f"BarnesHut was sized for n={self.n}, got {n}")
        return n

    @property
    def handle(self):
        return self._h

    def build(self, xm: torch.Tensor) -> None:
        self._last_n = self._n(xm)
        _lib.call("gb_bh_build", self._h, ptr(xm, "xm"), self._last_n, stream_handle(self.device))

    def accel(self, acc: torch.Tensor, accumulate: bool = False, phi=None) -> torch.Tensor:
        """Tree accelerations of the last build; with phi ((n,) float32
        device tensor) the traversal also writes the tree potential (the
        monopole terms of the accepted nodes, without G)."""
        flags = _lib.GB_ACCUMULATE if accumulate else 0
        if phi is None:
            _lib.call("gb_bh_accel", self._h, ptr(acc, "acc"), self.theta, self.eps2, self.G,
                      self.max_stack, flags, stream_handle(self.device))
        else:
            _lib.call("gb_bh_accel_phi", self._h, ptr(acc, "acc"), ptr(phi, "phi", rows4=False),
                      self.theta, self.eps2, self.G, self.max_stack, flags, stream_handle(self.device))
        return acc

    def accel_range(self, acc: torch.Tensor, s0: int, ns: int, accumulate: bool = False,
                    phi=None) -> torch.Tensor:
        """Tree accelerations of the last build for the targets at key-order
        positions s0 .. s0 + ns - 1 only, written at their particle indices
        of acc (and phi); bit-identical to those of accel()."""
        flags = _lib.GB_ACCUMULATE if accumulate else 0
        _lib.call("gb_bh_accel_range", self._h, ptr(acc, "acc"),
                  None if phi is None else ptr(phi, "phi", rows4=False), int(s0), int(ns),
                  self.theta, self.eps2, self.G, self.max_stack, flags, stream_handle(self.device))
        return acc

    def compute(self, *args, accumulate: bool = False, count_work: bool = False,
                check: bool = False, phi=None):
        """acc <- tree accelerations (core/solvers/barnes_hut.py:242-259).
        Call forms: ``compute(pos_field, mass_field, acc_field)``, the
        reference's (fields, numpy arrays or tensors; acc filled in place),
        or ``compute(xm, acc)`` on (n, 4) float32 device records.
        count_work adds the traversal work counters to diag() (a slightly
        slower kernel variant); check waits for the call and raises
        GravityError on failures counted since the last checked call (see
        the ``check`` constructor argument); phi ((n,) float32 device
        tensor, record form only) receives the tree potential."""
        if len(args) == 3:
            pos, mass, acc_out = args
            dev = pick_device(pos, mass, acc_out)
            xm = empty4(self.n, dev)
            xm[:, :3] = field_values(pos, dev)[: self.n].reshape(self.n, 3)
            xm[:, 3] = field_values(mass, dev)[: self.n].reshape(self.n)
            acc = empty4(self.n, dev)
            if accumulate:
                acc[:, :3] = field_values(acc_out, dev)[: self.n].reshape(self.n, 3)
            self._compute(xm, acc, accumulate, count_work, check)
            write_rows(acc_out, acc[:, :3])
            return acc_out
        xm, acc = args
        return self._compute(xm, acc, accumulate, count_work, check, phi)

    def _compute(self, xm, acc, accumulate, count_work, check=False, phi=None):
        self._last_n = self._n(xm)
        flags = ((_lib.GB_ACCUMULATE if accumulate else 0) | (_lib.GB_COUNT_WORK if count_work else 0)
                 | (_lib.GB_CHECK if check else 0))
        if phi is not None:
            _lib.call("gb_bh_build", self._h, ptr(xm, "xm"), self._last_n, stream_handle(self.device))
            _lib.call("gb_bh_accel_phi", self._h, ptr(acc, "acc"), ptr(phi, "phi", rows4=False),
                      self.theta, self.eps2, self.G, self.max_stack, flags, stream_handle(self.device))
            return acc
        _lib.call("gb_bh_compute", self._h, ptr(xm, "xm"), ptr(acc, "acc"), self._last_n,
                  self.theta, self.eps2, self.G, self.max_stack, flags, stream_handle(self.device))
        return acc

    def kdk(self, xm, vel, acc, dt: float, nsteps: int = 1, phi=None) -> None:
        """nsteps KDK leapfrog steps with tree forces, in place; with phi
        the last step also writes the tree potential of the final
        positions."""
        self._last_n = self._n(xm)
        if phi is None:
            _lib.call("gb_bh_kdk", self._h, ptr(xm, "xm"), ptr(vel, "vel"), ptr(acc, "acc"),
                      self._n(xm), self.theta, self.eps2, self.G, float(dt), int(nsteps),
                      self.max_stack, stream_handle(self.device))
        else:
            _lib.call("gb_bh_kdk_phi", self._h, ptr(xm, "xm"), ptr(vel, "vel"), ptr(acc, "acc"),
                      ptr(phi, "phi", rows4=False), self._n(xm), self.theta, self.eps2, self.G,
                      float(dt), int(nsteps), self.max_stack, stream_handle(self.device))

    def energies_from_phi(self, xm, vel, phi) -> tuple[float, float, float]:
        """(KE, PE, KE+PE) in FP64 from a tree potential phi."""
        if self._out3 is None:  # pinned host memory: the call copies and waits
            self._out3 = torch.zeros(3, dtype=torch.float64).pin_memory()
        _lib.call("gb_bh_energy", self._h, ptr(xm, "xm"), ptr(vel, "vel"),
                  ptr(phi, "phi", rows4=False), xm.shape[0], self.G, self._out3.data_ptr(),
                  stream_handle(self.device))
        e = self._out3.tolist()
        return e[0], e[1], e[2]

    def export(self, name: str) -> np.ndarray:
        """One array of the last build in the reference's layout."""
        what, dt, mult, off = EXPORTS[name]
        n = self._last_n
        count = mult * n + off
        shape = (count, 3) if name in ("com", "nmin", "nmax") else (count,)
        out = torch.empty(shape, dtype=_TORCH[dt], device=self.device)
        _lib.call("gb_bh_export", self._h, what, out.data_ptr(), stream_handle(self.device))
        a = out.cpu().numpy()
        return a.view(np.uint64) if dt is np.uint64 else a

    def tree_arrays(self) -> dict:
        return {k: self.export(k) for k in EXPORTS}

    def set_graph(self, on: bool = True) -> None:
        """kdk() replays one captured step as a CUDA graph (identical
        results, fewer launches)."""
        _lib.call("gb_bh_set_graph", self._h, 1 if on else 0)

    def set_traversal(self, targets_per_lane: int) -> None:
        """Traversal shape: 1 or 2 targets per lane, warp-coherent; 0
        per-lane walks; -1 (default) per lane below 131,072 particles and
        warp-coherent from there.  Results are bit-identical across these
        shapes.  3 (opt-in): group walk, each group of up to 32
        key-consecutive targets (one subtree) shares the node set its
        bounding box accepts under the reference's test: every target sums
        a refinement of its own node set, so the error is no larger, but
        the results are not bit-identical to the per-particle shapes and
        the max_stack rule does not apply."""
        _lib.call("gb_bh_set_traversal", self._h, int(targets_per_lane))

    # -- measurement hooks
    STAGES = ("keys", "sort", "build", "summaries", "traverse")

    def timing(self, enable: bool = True) -> None:
        """Record CUDA events at stage boundaries of every build/step."""
        _lib.call("gb_bh_timing", self._h, 1 if enable else 0)

    def stage_times(self) -> tuple[dict, int]:
        """(summed ms per stage, steps) since the last call (synchronises)."""
        ms = (ctypes.c_float * len(self.STAGES))()
        steps = ctypes.c_int()
        _lib.call("gb_bh_stage_times", self._h, ms, ctypes.byref(steps))
        return {k: float(ms[i]) for i, k in enumerate(self.STAGES)}, int(steps.value)

    def launch_count(self) -> int:
        return int(_lib.load().gb_bh_launch_count(self._h))

    def diag(self, reset: bool = False) -> dict:
        d = _lib.Diag()
        _lib.call("gb_bh_diag", self._h, ctypes.byref(d), 1 if reset else 0)
        return d.as_dict()
