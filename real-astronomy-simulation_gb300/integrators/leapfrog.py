"""Leapfrog halves on the GB300 (host side of gb_kick / gb_drift).

Mirrors core/integrators/leapfrog.py:11-22 with the reference's argument
lists, ``kick(vel, acc, n, dt_half)`` and ``drift(pos, vel, n, dt)``, on the
Engine's fields (``engine.vel``, ``engine.acc``, ``engine.pos``) or (n, 4)
float32 device records.  The Engine itself fuses both into the force pass;
these serve callers that step outside it.
"""
from __future__ import annotations

import torch

from .. import _lib
from .._dev import FieldView, stream_handle


def _records(x, name: str) -> torch.Tensor:
    """The (n, 4) float32 device buffer behind a field or record tensor."""
    t = x._buf if isinstance(x, FieldView) else x
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dim() == 2 and t.shape[1] == 4
            and t.dtype == torch.float32 and t.is_contiguous()):
        raise ValueError(f"{name} must be an Engine field or a contiguous (n, 4) float32 CUDA tensor")
    return t


def kick(vel, acc, n: int, dt_half: float) -> None:
    """vel[:n] += acc[:n] * dt_half (core/integrators/leapfrog.py:11-15)."""
    v, a = _records(vel, "vel"), _records(acc, "acc")
    _lib.call("gb_kick", v.data_ptr(), a.data_ptr(), int(n), float(dt_half), stream_handle(v.device))


def drift(pos, vel, n: int, dt: float) -> None:
    """pos[:n] += vel[:n] * dt (core/integrators/leapfrog.py:18-22); pos is
    the Engine's pos field or the (n, 4) records, whose mass column stays."""
    x, v = _records(pos, "pos"), _records(vel, "vel")
    _lib.call("gb_drift", x.data_ptr(), v.data_ptr(), int(n), float(dt), stream_handle(x.device))
