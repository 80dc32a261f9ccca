"""Analytic galaxy potential added after self-gravity (host side of
gb_analytic_acc, gb_direct_acc_ext and gb_bh_accel_ext).

Mirrors the force pass of the reference's living-galaxy and gas-disk
engines:

* ``grav_analytic(xm, acc, n, M_d, a, b, M_h, a_h, is_hernquist, smbh_mass)``
  (core/living_galaxy_engine.py:124-151) and its copy ``add_analytic``
  (core/gas_disk_engine.py:54-81): acc += the analytic acceleration;
* ``add_grav_ext(xm, acc, n, eps2, M_d, ...)`` (core/gas_disk_engine.py:
  20-51): acc += direct self-gravity + the analytic acceleration, in one
  direct-sum launch whose result pass adds the potential;
* ``tree_forces_ext`` for the tree branch (BarnesHut.compute + add_field /
  add_acc + add_analytic / grav_analytic, core/gas_disk_engine.py:216-225,
  core/living_galaxy_engine.py:1013-1027), with the potential added in the
  traversal's result pass.

Positions and masses are the (n, 4) float32 ``xm`` tensor, accelerations
(n, 4) float32.  The potential is evaluated in FP32 with G folded into the
masses; the engines' ``pot`` dict (keys M_d, a, b, M_h, a_h and optionally
is_hernquist, smbh_mass) converts with ``Potential.from_dict``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from .. import _lib
from .._dev import ptr, stream_handle
from ..units import G as G_DEFAULT
from .gravity import _solver_for


@dataclass(frozen=True)
class Potential:
    M_d: float
    a: float
    b: float
    M_h: float
    a_h: float
    is_hernquist: int = 0
    smbh_mass: float = 0.0

    @classmethod
    def from_dict(cls, pot: dict) -> "Potential":
        return cls(float(pot["M_d"]), float(pot["a"]), float(pot["b"]), float(pot["M_h"]),
                   float(pot["a_h"]), int(pot.get("is_hernquist", 0)), float(pot.get("smbh_mass", 0.0)))

    def to_c(self) -> _lib.Potential:
        return _lib.Potential(self.M_d, self.a, self.b, self.M_h, self.a_h, self.smbh_mass,
                              int(self.is_hernquist), 0)


def analytic_acc(xm: torch.Tensor, acc: torch.Tensor, pot: Potential, G: float = G_DEFAULT,
                 accumulate: bool = True) -> torch.Tensor:
    """acc += (or =) the potential's acceleration at every particle."""
    c = pot.to_c()
    _lib.call("gb_analytic_acc", ptr(xm, "xm"), ptr(acc, "acc"), xm.shape[0], float(G),
              ctypes.addressof(c), _lib.GB_ACCUMULATE if accumulate else 0, stream_handle(xm.device))
    return acc


def direct_acc_ext(solver, xm: torch.Tensor, acc: torch.Tensor, G: float, eps2: float,
                   pot: Potential | None, accumulate: bool = True, plain: bool = False) -> torch.Tensor:
    """acc (+)= direct self-gravity + the potential with one gb_direct handle
    (the potential is added in the pass that writes the results)."""
    c = pot.to_c() if pot is not None else None
    flags = (_lib.GB_ACCUMULATE if accumulate else 0) | (_lib.GB_PLAIN_FP32 if plain else 0)
    _lib.call("gb_direct_acc_ext", solver.handle, ptr(xm, "xm"), ptr(acc, "acc"), xm.shape[0],
              float(G), float(eps2), ctypes.addressof(c) if c is not None else None, flags,
              stream_handle(xm.device))
    return acc


def tree_forces_ext(bh, xm: torch.Tensor, acc: torch.Tensor, pot: Potential | None,
                    accumulate: bool = True) -> torch.Tensor:
    """Tree build + traversal with the potential added in the traversal's
    result pass: acc (+)= tree self-gravity + the potential."""
    bh.build(xm)
    c = pot.to_c() if pot is not None else None
    _lib.call("gb_bh_accel_ext", bh.handle, ptr(acc, "acc"), bh.theta, bh.eps2, bh.G, bh.max_stack,
              ctypes.addressof(c) if c is not None else None,
              _lib.GB_ACCUMULATE if accumulate else 0, stream_handle(xm.device))
    return acc


# ----------------------------------------------- reference-named mirrors
def grav_analytic(xm, acc, n, M_d, a, b, M_h, a_h, is_hernquist=0, smbh_mass=0.0, G=G_DEFAULT):
    """acc[:n] += analytic disk + halo (+ point mass) acceleration
    (core/living_galaxy_engine.py:124-151)."""
    pot = Potential(M_d, a, b, M_h, a_h, int(is_hernquist), smbh_mass)
    analytic_acc(xm[:n], acc[:n], pot, G, accumulate=True)


add_analytic = grav_analytic  # core/gas_disk_engine.py:54-81 (same terms)


def add_grav_ext(xm, acc, n, eps2, M_d, a, b, M_h, a_h, is_hernquist=0, smbh_mass=0.0, G=G_DEFAULT):
    """acc[:n] += softened direct self-gravity + the analytic potential
    (core/gas_disk_engine.py:20-51)."""
    pot = Potential(M_d, a, b, M_h, a_h, int(is_hernquist), smbh_mass)
    direct_acc_ext(_solver_for(xm), xm[:n], acc[:n], G, eps2, pot, accumulate=True)
