"""ctypes binding of the C ABI in include/gbgrav.h (libgbgrav.so).

The library must have been built (``_buildlib.build()`` / ``build()`` in
``__graft_entry__``).  There is no fallback: if it is missing, every entry
point raises.
"""
from __future__ import annotations

import ctypes
import os

from . import _buildlib

P = ctypes.c_void_p
I32 = ctypes.c_int
I64 = ctypes.c_int64
F32 = ctypes.c_float
F64 = ctypes.c_double

GB_OK = 0
GB_EINVAL = 1
GB_ENOMEM = 2
GB_ESTACK = 3
GB_ETIMEOUT = 4
GB_ECUDA = 5
GB_ENOTREADY = 6

GB_ACCUMULATE = 0x1
GB_PLAIN_FP32 = 0x2
GB_COUNT_WORK = 0x4
GB_USE_GRAPH = 0x8
GB_CHECK = 0x10

_STATUS = {GB_EINVAL: "GB_EINVAL", GB_ENOMEM: "GB_ENOMEM", GB_ESTACK: "GB_ESTACK",
           GB_ETIMEOUT: "GB_ETIMEOUT", GB_ECUDA: "GB_ECUDA",
           GB_ENOTREADY: "GB_ENOTREADY"}


class GravityError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, func: str, msg: str):
        self.status = status
        super().__init__(f"{func}: {_STATUS.get(status, status)}: {msg}")


class Diag(ctypes.Structure):
    _fields_ = [("stack_drops", ctypes.c_uint64), ("stack_overflow", ctypes.c_uint64),
                ("nonfinite", ctypes.c_uint64), ("bad_tree", ctypes.c_uint64),
                ("warp_node_reads", ctypes.c_uint64), ("warp_root_reads", ctypes.c_uint64),
                ("lane_interactions", ctypes.c_uint64), ("lane_tests", ctypes.c_uint64),
                ("wait_timeouts", ctypes.c_uint64)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


# name -> (restype, argtypes)
class Potential(ctypes.Structure):
    """gb_potential_t: the analytic galaxy potential (Miyamoto-Nagai disk,
    Hernquist or Plummer halo, optional central point mass)."""
    _fields_ = [("M_d", ctypes.c_double), ("a", ctypes.c_double), ("b", ctypes.c_double),
                ("M_h", ctypes.c_double), ("a_h", ctypes.c_double), ("smbh_mass", ctypes.c_double),
                ("is_hernquist", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class GridInfo(ctypes.Structure):
    """gb_grid_info_t: the geometry of the last neighbour-grid rebuild."""
    _fields_ = [("ngas", ctypes.c_int64), ("n_cells", ctypes.c_int64), ("nx", ctypes.c_int32),
                ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("status", ctypes.c_int32),
                ("lo", ctypes.c_double * 3), ("cell", ctypes.c_double), ("inv_cell", ctypes.c_double)]


SIGNATURES = {
    "gb_last_error_string": (ctypes.c_char_p, []),
    "gb_version": (I32, []),
    "gb_direct_create": (I32, [ctypes.POINTER(P), I64]),
    "gb_direct_destroy": (I32, [P]),
    "gb_direct_set_tiles": (I32, [P, I32, I32, I32]),
    "gb_direct_set_variant": (I32, [P, I32]),
    "gb_direct_set_sym_band": (I32, [P, I64]),
    "gb_direct_acc": (I32, [P, P, P, I64, F32, F32, I32, P]),
    "gb_direct_kdk": (I32, [P, P, P, P, I64, F32, F32, F32, I64, I32, P]),
    "gb_direct_phi": (I32, [P, P, P, I64, F32, I32, P]),
    "gb_energy": (I32, [P, P, P, I64, F32, F32, P, P]),
    "gb_direct_acc_phi": (I32, [P, P, P, P, I64, F32, F32, I32, P]),
    "gb_direct_acc_range": (I32, [P, P, I64, I64, I64, P, P, F32, F32, I32, P]),
    "gb_direct_kdk_phi": (I32, [P, P, P, P, P, I64, F32, F32, F32, I64, I32, P]),
    "gb_energy_phi": (I32, [P, P, P, P, I64, F32, P, P]),
    "gb_direct_acc_fp64": (I32, [P, I64, P, I64, F64, F64, P, P]),
    "gb_direct_diag": (I32, [P, ctypes.POINTER(Diag), I32]),
    "gb_direct_launch_count": (ctypes.c_uint64, [P]),
    "gb_calib_fp32": (I32, [P, I32, I32, ctypes.POINTER(F64), P]),
    "gb_direct_acc_noalloc": (I32, [P, P, I64, F32, F32, I32, P]),
    "gb_bh_create": (I32, [ctypes.POINTER(P), I64, I32]),
    "gb_bh_destroy": (I32, [P]),
    "gb_bh_build": (I32, [P, P, I64, P]),
    "gb_bh_accel": (I32, [P, P, F32, F32, F32, I32, I32, P]),
    "gb_bh_compute": (I32, [P, P, P, I64, F32, F32, F32, I32, I32, P]),
    "gb_bh_kdk": (I32, [P, P, P, P, I64, F32, F32, F32, F32, I64, I32, P]),
    "gb_bh_accel_phi": (I32, [P, P, P, F32, F32, F32, I32, I32, P]),
    "gb_bh_accel_range": (I32, [P, P, P, I64, I64, F32, F32, F32, I32, I32, P]),
    "gb_bh_kdk_phi": (I32, [P, P, P, P, P, I64, F32, F32, F32, F32, I64, I32, P]),
    "gb_bh_energy": (I32, [P, P, P, P, I64, F32, P, P]),
    "gb_bh_export": (I32, [P, I32, P, P]),
    "gb_bh_diag": (I32, [P, ctypes.POINTER(Diag), I32]),
    "gb_bh_timing": (I32, [P, I32]),
    "gb_bh_set_traversal": (I32, [P, I32]),
    "gb_bh_stage_times": (I32, [P, ctypes.POINTER(F32), ctypes.POINTER(I32)]),
    "gb_bh_launch_count": (ctypes.c_uint64, [P]),
    "gb_batch_create": (I32, [ctypes.POINTER(P), P, I32]),
    "gb_batch_destroy": (I32, [P]),
    "gb_batch_set_tiles": (I32, [P, I32, I32, I32]),
    "gb_batch_set_variant": (I32, [P, I32]),
    "gb_batch_total": (I64, [P]),
    "gb_batch_acc": (I32, [P, P, P, F32, F32, I32, P]),
    "gb_batch_kdk": (I32, [P, P, P, P, F32, F32, F32, I64, I32, P]),
    "gb_batch_kdk_loop": (I32, [P, P, P, P, F32, F32, F32, I64, I32, P]),
    "gb_batch_launch_count": (ctypes.c_uint64, [P]),
    "gb_adjoint_step": (I32, [P, P, P, P, P, P, I64, F32, F32, F32, I32, P]),
    "gb_adjoint_set_variant": (I32, [P, I32]),
    "gb_analytic_acc": (I32, [P, P, I64, F32, P, I32, P]),
    "gb_direct_acc_ext": (I32, [P, P, P, I64, F32, F32, P, I32, P]),
    "gb_bh_accel_ext": (I32, [P, P, F32, F32, F32, I32, P, I32, P]),
    "gb_bh_set_graph": (I32, [P, I32]),
    "gb_bh_set_check": (I32, [P, I32]),
    "gb_sort_wait_probe": (I32, [I32, I32, P, P]),
    "gb_kick": (I32, [P, P, I64, F32, P]),
    "gb_drift": (I32, [P, P, I64, F32, P]),
    "gb_grid_create": (I32, [ctypes.POINTER(P), I64, F64]),
    "gb_grid_destroy": (I32, [P]),
    "gb_grid_max_cells": (I64, [P]),
    "gb_grid_rebuild": (I32, [P, P, P, P, P, P, P, P]),
    "gb_grid_launch_count": (ctypes.c_uint64, [P]),
}

_lib = None


def lib_path() -> str:
    return _buildlib.LIB


def load():
    """Load libgbgrav.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build the CUDA engine first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def call(name: str, *args) -> int:
    """Call an int-returning entry point; raise GravityError on failure."""
    L = load()
    st = getattr(L, name)(*args)
    if st != GB_OK:
        msg = L.gb_last_error_string()
        raise GravityError(st, name, msg.decode() if msg else "")
    return st
