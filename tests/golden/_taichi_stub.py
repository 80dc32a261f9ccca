"""Minimal stand-in for the ``taichi`` module, used ONLY to execute the
reference's own hot-path Python source on the host when generating golden
fixtures (``gen_golden.py``).  Taichi itself is not installable offline.

Under this stub a ``@ti.kernel`` / ``@ti.func`` body runs as ordinary serial
Python: the outermost ``for`` loop (parallel in Taichi) runs in index order,
fields are numpy arrays, ``ti.Vector`` is a float64 numpy vector.  Every
kernel on the path is data-parallel over its outer index with no cross-index
dependence, except ``_accumulate`` (float64 atomics; addition order differs
from a GPU run only at the last-bit level) and the scalar energy reductions.

``ti.atomic_*`` cannot update a numpy element passed by value; ``gen_golden``
therefore rewrites the three atomic calls in ``_accumulate`` textually into
in-place updates before running it (see ``rewrite_atomics``).
"""
from __future__ import annotations

import math
import re
import sys
import types

import numpy as np


class Field(np.ndarray):
    """numpy array with Taichi's host-transfer methods; a row of a vector
    field also has Taichi's ``.x/.y/.z`` and ``.norm()``."""

    def from_numpy(self, arr):
        self[...] = np.asarray(arr).reshape(self.shape)

    def to_numpy(self):
        return np.array(self)

    @property
    def x(self):
        return np.float64(self[0])

    @property
    def y(self):
        return np.float64(self[1])

    @property
    def z(self):
        return np.float64(self[2])

    def norm(self):
        x, y, z = (np.float64(self[k]) for k in range(3))
        return np.sqrt(x * x + y * y + z * z)


def _field(dtype, shape):
    np_dt = {"f64": np.float64, "f32": np.float32, "i32": np.int32,
             "i64": np.int64}[dtype]
    shape = (shape,) if isinstance(shape, int) else tuple(shape)
    return np.zeros(shape, np_dt).view(Field)


class _Vector:
    def __call__(self, values, dt=None):
        return np.array(values, dtype=np.float64)

    @staticmethod
    def field(k, dtype, shape):
        shape = (shape,) if isinstance(shape, int) else tuple(shape)
        return _field(dtype, shape + (k,))


def _identity(fn=None, **_kw):
    if fn is None:
        return lambda f: f
    return fn


def make_module() -> types.ModuleType:
    ti = types.ModuleType("taichi")
    ti.f64, ti.f32, ti.i32, ti.i64 = "f64", "f32", "i32", "i64"
    ti.cuda, ti.vulkan, ti.cpu, ti.gpu = "cuda", "vulkan", "cpu", "gpu"
    ti.kernel = _identity
    ti.func = _identity
    ti.data_oriented = _identity
    ti.template = lambda: None
    ti.static = lambda x: x
    ti.sqrt = math.sqrt
    ti.max = max
    ti.min = min
    ti.init = lambda **kw: None
    ti.Vector = _Vector()
    ti.field = lambda dtype, shape: _field(dtype, shape)

    # Integer "constructors" used as ti.i64(1) << 62 in the reference.
    class _IntType(str):
        def __call__(self, v):
            return np.int64(v) if self == "i64" else np.int32(v)

    ti.i64 = _IntType("i64")
    ti.i32 = _IntType("i32")
    return ti


def install() -> types.ModuleType:
    ti = make_module()
    sys.modules["taichi"] = ti
    return ti


_ATOMIC = re.compile(r"ti\.atomic_(add|min|max)\((.+?),\s*(.+)\)\s*$")


def rewrite_atomics(src: str) -> str:
    """Turn ``ti.atomic_add(X, v)`` into ``X += v`` and atomic min/max into
    ``X = min(X, v)`` / ``X = max(X, v)``, line by line."""
    out = []
    for line in src.splitlines():
        m = _ATOMIC.search(line)
        if m:
            op, target, val = m.groups()
            indent = line[: m.start()]
            if op == "add":
                line = f"{indent}{target} += {val}"
            else:
                line = f"{indent}{target} = {op}({target}, {val})"
        out.append(line)
    return "\n".join(out) + "\n"
