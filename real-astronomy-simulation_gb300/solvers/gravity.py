"""Direct N^2 gravity on the GB300 (host side of gb_direct_*).

Mirrors core/solvers/gravity.py:13-57 of the reference:

* ``compute_acc_direct(xm, acc, n, grav, eps2)``  (gravity.py:13-26)
* ``kinetic_energy(vel, xm, n)``                  (gravity.py:29-36)
* ``potential_energy(xm, n, grav, eps2)``          (gravity.py:39-57)

Positions and masses travel together as one (n, 4) float32 ``xm`` tensor;
accelerations and velocities are (n, 4) float32 tensors.  The arithmetic is
FP32 with Kahan-compensated accumulation (FP64 for the energy reductions).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib
from .._dev import empty4, field_values, pick_device, ptr, require_cuda, stream_handle, write_rows


class DirectGravity:
    """Owns a gb_direct handle (scratch for up to ``n_max`` particles)."""

    def __init__(self, n_max: int, device=None, tiles=None):
        self.device = require_cuda(device)
        self.n_max = int(n_max)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("gb_direct_create", ctypes.byref(h), self.n_max)
        self._h = h
        self._out3 = torch.zeros(3, dtype=torch.float64, device=self.device)
        if tiles is not None:
            self.set_tiles(*tiles)

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().gb_direct_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_tiles(self, k: int, warps: int, ctas_per_sm: int = 0, packed: int | None = None):
        _lib.call("gb_direct_set_tiles", self._h, int(k), int(warps), int(ctas_per_sm))
        if packed is not None:
            _lib.call("gb_direct_set_variant", self._h, int(packed))

    def set_variant(self, variant: int):
        """Force-pass form: 0 scalar per target (default), 1 packed per
        target, 2 symmetric (each unordered pair once, both particles
        updated; its tile-pair scratch is bounded by running large systems in
        bands, see set_sym_band).  phi() and energies() follow the variant."""
        _lib.call("gb_direct_set_variant", self._h, int(variant))

    def set_sym_band(self, nbytes: int):
        """Slot bytes per band of the symmetric pass (default 1 GiB); larger
        systems run in bands of tile rows."""
        _lib.call("gb_direct_set_sym_band", self._h, int(nbytes))

    # -- compute
    def acc(self, xm, acc, G, eps2, accumulate=False, plain=False):
        flags = (_lib.GB_ACCUMULATE if accumulate else 0) | (_lib.GB_PLAIN_FP32 if plain else 0)
        n = xm.shape[0]
        _lib.call("gb_direct_acc", self._h, ptr(xm, "xm"), ptr(acc, "acc"), n,
                  float(G), float(eps2), flags, stream_handle(self.device))
        return acc

    def acc_phi(self, xm, acc, phi, G, eps2, plain=False):
        """acc() that also writes the potential sums of the same positions
        into phi ((n,) float32 device tensor, without G) from the same pass."""
        n = xm.shape[0]
        _lib.call("gb_direct_acc_phi", self._h, ptr(xm, "xm"), ptr(acc, "acc"),
                  ptr(phi, "phi", rows4=False), n, float(G), float(eps2),
                  _lib.GB_PLAIN_FP32 if plain else 0, stream_handle(self.device))
        return acc

    def acc_range(self, xm, n, t0, nt, acc, G, eps2, phi=None, accumulate=False, plain=False):
        """Accelerations of targets t0 .. t0 + nt - 1 from the first n
        records of xm into acc[:nt] (and their potential sums into phi[:nt]
        when phi is given): one rank's slice of the target loop."""
        if xm.shape[0] < n or acc.shape[0] < nt or (phi is not None and phi.shape[0] < nt):
            raise ValueError("acc_range: buffers shorter than n / nt")
        flags = (_lib.GB_ACCUMULATE if accumulate else 0) | (_lib.GB_PLAIN_FP32 if plain else 0)
        _lib.call("gb_direct_acc_range", self._h, ptr(xm, "xm"), int(n), int(t0), int(nt),
                  ptr(acc, "acc"), None if phi is None else ptr(phi, "phi", rows4=False),
                  float(G), float(eps2), flags, stream_handle(self.device))
        return acc

    def kdk(self, xm, vel, acc, G, eps2, dt, nsteps=1, plain=False, graph=False, phi=None):
        """nsteps fused KDK steps in place; graph=True replays captured
        steps as CUDA graphs (identical results, fewer launches).  With phi
        ((n,) float32 device tensor) the last step's force pass also writes
        the potential sums of the final positions."""
        n = xm.shape[0]
        flags = (_lib.GB_PLAIN_FP32 if plain else 0) | (_lib.GB_USE_GRAPH if graph else 0)
        if phi is None:
            _lib.call("gb_direct_kdk", self._h, ptr(xm, "xm"), ptr(vel, "vel"), ptr(acc, "acc"),
                      n, float(G), float(eps2), float(dt), int(nsteps), flags, stream_handle(self.device))
        else:
            _lib.call("gb_direct_kdk_phi", self._h, ptr(xm, "xm"), ptr(vel, "vel"), ptr(acc, "acc"),
                      ptr(phi, "phi", rows4=False), n, float(G), float(eps2), float(dt), int(nsteps),
                      flags, stream_handle(self.device))

    def phi(self, xm, eps2, out=None, plain=False):
        n = xm.shape[0]
        if out is None:
            out = torch.empty(n, dtype=torch.float32, device=xm.device)
        _lib.call("gb_direct_phi", self._h, ptr(xm, "xm"), ptr(out, "phi", rows4=False), n,
                  float(eps2), _lib.GB_PLAIN_FP32 if plain else 0, stream_handle(self.device))
        return out

    def energies_async(self, xm, vel, G, eps2) -> torch.Tensor:
        """(KE, PE, KE+PE) as a float64 device tensor (no host sync)."""
        _lib.call("gb_energy", self._h, ptr(xm, "xm"), ptr(vel, "vel"), xm.shape[0],
                  float(G), float(eps2), ptr(self._out3, "out3", torch.float64, rows4=False),
                  stream_handle(self.device))
        return self._out3

    def _host3(self):
        """Pinned host buffer the energy calls copy their three sums into
        (the call then waits for its stream)."""
        if getattr(self, "_out3_host", None) is None:
            self._out3_host = torch.zeros(3, dtype=torch.float64).pin_memory()
        return self._out3_host

    def energies(self, xm, vel, G, eps2):
        out = self._host3()
        _lib.call("gb_energy", self._h, ptr(xm, "xm"), ptr(vel, "vel"), xm.shape[0],
                  float(G), float(eps2), out.data_ptr(), stream_handle(self.device))
        e = out.tolist()
        return e[0], e[1], e[2]

    def energies_from_phi(self, xm, vel, phi, G):
        """(KE, PE, KE+PE) from potential sums phi the force pass already
        produced: only the O(n) FP64 reductions run (one launch, a 24-byte
        copy to pinned host memory)."""
        out = self._host3()
        _lib.call("gb_energy_phi", self._h, ptr(xm, "xm"), ptr(vel, "vel"),
                  ptr(phi, "phi", rows4=False), xm.shape[0], float(G), out.data_ptr(),
                  stream_handle(self.device))
        e = out.tolist()
        return e[0], e[1], e[2]

    def launch_count(self) -> int:
        return int(_lib.load().gb_direct_launch_count(self._h))

    def diag(self, reset=False) -> dict:
        d = _lib.Diag()
        _lib.call("gb_direct_diag", self._h, ctypes.byref(d), 1 if reset else 0)
        return d.as_dict()


def acc_fp64_targets(xm: torch.Tensor, targets, G: float, eps2: float) -> np.ndarray:
    """FP64 accelerations of the listed particles, computed on the device
    (gb_direct_acc_fp64); returns a (len(targets), 3) float64 array."""
    t = torch.as_tensor(np.asarray(targets, dtype=np.int64), device=xm.device)
    out = torch.empty((t.numel(), 3), dtype=torch.float64, device=xm.device)
    if t.numel():
        _lib.call("gb_direct_acc_fp64", ptr(xm, "xm"), xm.shape[0],
                  ptr(t, "targets", torch.int64, rows4=False), t.numel(), float(G), float(eps2),
                  ptr(out, "acc_out", torch.float64, rows4=False), stream_handle(xm.device))
    return out.cpu().numpy()


_CACHE: dict = {}


def _solver_for(xm: torch.Tensor) -> DirectGravity:
    key = xm.device.index
    s = _CACHE.get(key)
    if s is None or s.n_max < xm.shape[0]:
        s = DirectGravity(max(xm.shape[0], 1), xm.device)
        s.set_variant(2)  # the symmetric pass, as the Engine uses
        _CACHE[key] = s
    return s


def _pack(pos, mass, n) -> torch.Tensor:
    """(n, 4) float32 device records from separate position and mass fields."""
    dev = pick_device(pos, mass)
    xm = empty4(n, dev)
    xm[:, :3] = field_values(pos, dev)[:n].reshape(n, 3)
    xm[:, 3] = field_values(mass, dev)[:n].reshape(n)
    return xm


def _is_records(x) -> bool:
    return isinstance(x, torch.Tensor) and x.dim() == 2 and x.shape[1] == 4


def compute_acc_direct(*args):
    """acc[:n] = G sum_j m_j d_ij / (|d_ij|^2 + eps2)^{3/2}
    (core/solvers/gravity.py:13-26).  Two call forms:

    * ``compute_acc_direct(pos, mass, acc, n, grav, eps2)``, the reference's:
      pos / acc (n, 3) and mass (n,) as reference-style fields (``to_numpy``
      / ``from_numpy``), numpy arrays or torch tensors; acc is filled in
      place (rows 0..n-1);
    * ``compute_acc_direct(xm, acc, n, grav, eps2)`` on (n, 4) float32 device
      records (no copies)."""
    if len(args) == 6:
        pos, mass, acc, n, grav, eps2 = args
        n = int(n)
        xm = _pack(pos, mass, n)
        out = empty4(n, xm.device)
        _solver_for(xm).acc(xm, out, grav, eps2)
        write_rows(acc, out[:, :3])
        return
    xm, acc, n, grav, eps2 = args
    xm_n = xm[:n] if n != xm.shape[0] else xm
    acc_n = acc[:n] if n != acc.shape[0] else acc
    _solver_for(xm).acc(xm_n, acc_n, grav, eps2)


def kinetic_energy(vel, mass, n, grav=1.0, eps2=1.0):
    """1/2 sum m |v|^2 in FP64 (core/solvers/gravity.py:29-36).  ``mass``
    is the reference's (n,) mass field or, with device records, the (n, 4)
    ``xm`` tensor; vel is a reference-style field, array or tensor."""
    n = int(n)
    xm = mass[:n] if _is_records(mass) else _pack(torch.zeros((n, 3)), mass, n)
    v = field_values(vel, xm.device)[:n]
    v4 = empty4(n, xm.device)
    v4[:, :3] = v[:, :3] if v.dim() == 2 else v.reshape(n, 3)
    return _solver_for(xm).energies(xm, v4, grav, eps2)[0]


def potential_energy(*args, vel=None):
    """-1/2 G sum_i m_i sum_{j != i} m_j / sqrt(r^2 + eps2)
    (core/solvers/gravity.py:39-57); FP32 pair sums, FP64 reduction.  Call
    forms: ``potential_energy(pos, mass, n, grav, eps2)`` (the reference's)
    or ``potential_energy(xm, n, grav, eps2)`` on device records."""
    if len(args) == 5:
        pos, mass, n, grav, eps2 = args
        xm = _pack(pos, mass, int(n))
    else:
        xm, n, grav, eps2 = args
        xm = xm[:n]
    return _solver_for(xm).energies(xm, torch.zeros_like(xm), grav, eps2)[1]
