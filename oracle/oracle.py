"""ORACLE — test infrastructure only (what the tests compare against, never
the product).

Python front end of the float64 CPU restatement of the reference's hot path
(``gboracle.c``), plus a numpy restatement of the reference's Morton keys.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module.  Pinned against the golden fixtures generated from the
reference's own code (``tests/golden``).

Every function follows a reference function line by line:

* ``direct_acc``          core/solvers/gravity.py:13-26
* ``kinetic_energy``      core/solvers/gravity.py:29-36
* ``potential_energy``    core/solvers/gravity.py:39-57
* ``kdk_direct``          core/integrators/leapfrog.py:11-22, core/engine.py:108-116
* ``morton_codes``        core/solvers/barnes_hut.py:27-46 (C and numpy)
* ``stable_argsort``      core/solvers/barnes_hut.py:247
* ``build_radix``         core/solvers/barnes_hut.py:50-121
* ``summaries``           core/solvers/barnes_hut.py:124-177
* ``traverse``            core/solvers/barnes_hut.py:180-217
* ``traverse_phi``        the same walk's monopole potential (gravity.py:47-55 on its node set)
* ``group_walk``          the walk with the acceptance test applied to a group's box (:204-210)
* ``bh_compute``          core/solvers/barnes_hut.py:242-259
* ``analytic_acc``        core/living_galaxy_engine.py:124-151, core/gas_disk_engine.py:54-81
* ``grav_ext_acc``        core/gas_disk_engine.py:20-51
* ``grid_rebuild``        core/solvers/neighbor_grid.py:49-136
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libgboracle.so")
SRC = os.path.join(HERE, "gboracle.c")

_lib = None


def build(force: bool = False) -> str:
    """Compile gboracle.c into oracle/_build/libgboracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _declare(_lib)
    return _lib


P = ctypes.c_void_p
I64 = ctypes.c_int64
I32 = ctypes.c_int
D = ctypes.c_double


def _declare(L):
    L.orc_max_threads.restype = I32
    L.orc_direct_acc.argtypes = [P, P, P, I64, D, D]
    L.orc_direct_acc_targets.argtypes = [P, P, I64, P, I64, D, D, P]
    L.orc_phi_targets.argtypes = [P, P, I64, P, I64, D, P]
    L.orc_kinetic_energy.argtypes = [P, P, I64]
    L.orc_kinetic_energy.restype = D
    L.orc_potential_energy.argtypes = [P, P, I64, D, D]
    L.orc_potential_energy.restype = D
    L.orc_kdk_direct.argtypes = [P, P, P, P, I64, D, D, D, I64]
    L.orc_analytic_acc.argtypes = [P, P, I64, D, D, D, D, D, D, I32, D]
    L.orc_grid_rebuild.argtypes = [P, P, P, I64, D, I64, P, P, P, P, P]
    L.orc_grid_rebuild.restype = I64
    L.orc_grav_ext_acc.argtypes = [P, P, P, I64, D, D, D, D, D, D, D, I32, D]
    L.orc_morton.argtypes = [P, I64, I32, P, P, P]
    L.orc_stable_argsort_u64.argtypes = [P, I64, P]
    L.orc_build_radix.argtypes = [P, I32, P, P, P]
    L.orc_summaries.argtypes = [P, P, P, P, I32, P, P, P, P]
    L.orc_traverse.argtypes = [P, P, P, P, P, P, P, P, I32, D, D, I32, D, P,
                               I64, P]
    L.orc_traverse.restype = I64
    L.orc_traverse_phi.argtypes = [P, P, P, P, P, P, P, P, I32, D, D, I32, D, P,
                                   I64, P, P]
    L.orc_traverse_phi.restype = I64
    L.orc_group_walk.argtypes = [P, P, P, P, P, P, P, P, I32, I32, D, D, D, P, P]


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.reshape(shape) if shape is not None else a


def max_threads() -> int:
    return lib().orc_max_threads()


# ------------------------------------------------------------------ direct
def direct_acc(pos, mass, G, eps2, targets=None):
    pos = _f64(pos, (-1, 3))
    mass = _f64(mass, (-1,))
    n = pos.shape[0]
    if targets is None:
        out = np.empty((n, 3))
        lib().orc_direct_acc(_p(pos), _p(mass), _p(out), n, G, eps2)
        return out
    t = np.ascontiguousarray(targets, dtype=np.int64)
    out = np.empty((t.size, 3))
    lib().orc_direct_acc_targets(_p(pos), _p(mass), n, _p(t), t.size, G, eps2,
                                 _p(out))
    return out


def phi_targets(pos, mass, eps2, targets):
    pos = _f64(pos, (-1, 3))
    mass = _f64(mass, (-1,))
    t = np.ascontiguousarray(targets, dtype=np.int64)
    out = np.empty(t.size)
    lib().orc_phi_targets(_p(pos), _p(mass), pos.shape[0], _p(t), t.size, eps2,
                          _p(out))
    return out


def kinetic_energy(vel, mass):
    vel = _f64(vel, (-1, 3))
    mass = _f64(mass, (-1,))
    return lib().orc_kinetic_energy(_p(vel), _p(mass), vel.shape[0])


def potential_energy(pos, mass, G, eps2):
    pos = _f64(pos, (-1, 3))
    mass = _f64(mass, (-1,))
    return lib().orc_potential_energy(_p(pos), _p(mass), pos.shape[0], G, eps2)


def kdk_direct(pos, vel, acc, mass, G, eps2, dt, nsteps):
    """Returns (pos, vel, acc) after nsteps KDK steps (copies)."""
    pos = _f64(pos, (-1, 3)).copy()
    vel = _f64(vel, (-1, 3)).copy()
    acc = _f64(acc, (-1, 3)).copy()
    mass = _f64(mass, (-1,))
    lib().orc_kdk_direct(_p(pos), _p(vel), _p(acc), _p(mass), pos.shape[0], G,
                         eps2, dt, nsteps)
    return pos, vel, acc


# ------------------------------------------------------ analytic potential
def _pot_args(pot):
    return (float(pot["M_d"]), float(pot["a"]), float(pot["b"]), float(pot["M_h"]),
            float(pot["a_h"]), int(pot.get("is_hernquist", 0)), float(pot.get("smbh_mass", 0.0)))


def analytic_acc(pos, G, pot, acc=None):
    """acc + the analytic disk/halo/point-mass acceleration (grav_analytic,
    add_analytic); acc defaults to zero.  Returns a new (n, 3) array."""
    pos = _f64(pos, (-1, 3))
    out = np.zeros_like(pos) if acc is None else _f64(acc, (-1, 3)).copy()
    lib().orc_analytic_acc(_p(pos), _p(out), pos.shape[0], G, *_pot_args(pot))
    return out


def grav_ext_acc(pos, mass, G, eps2, pot, acc=None):
    """acc + direct self-gravity + the analytic potential (add_grav_ext)."""
    pos = _f64(pos, (-1, 3))
    mass = _f64(mass, (-1,))
    out = np.zeros_like(pos) if acc is None else _f64(acc, (-1, 3)).copy()
    lib().orc_grav_ext_acc(_p(pos), _p(mass), _p(out), pos.shape[0], G, eps2, *_pot_args(pot))
    return out


# ------------------------------------------------------ neighbour grid
def grid_rebuild(pos, h, is_star=None, min_radius=0.0, state=None):
    """NeighborGrid(n, min_radius).rebuild(pos, h, is_star) (or rebuild_all
    when is_star is None).  state: a previous result whose gsort/cell_start/
    geometry a rebuild without gas leaves in place.  Returns a dict with
    ngas, gsort, cell_start, dims, lo, inv_cell."""
    pos = _f64(pos, (-1, 3))
    n = pos.shape[0]
    h = _f64(h, (-1,))
    max_cells = max(64, 4 * n)
    if state is None:
        state = dict(gsort=np.zeros(max(n, 1), np.int32), cell_start=np.zeros(max_cells + 1, np.int32),
                     dims=np.ones(3, np.int64), lo=np.zeros(3), inv_cell=1.0)
    out = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in state.items()}
    star = None if is_star is None else np.ascontiguousarray(is_star, dtype=np.int32)
    dims = out["dims"]
    lo = out["lo"]
    inv = np.array([out["inv_cell"]], np.float64)
    ngas = lib().orc_grid_rebuild(_p(pos), _p(h), _p(star) if star is not None else None, n,
                                  float(min_radius), max_cells, _p(out["gsort"]), _p(out["cell_start"]),
                                  _p(dims), _p(lo), _p(inv))
    out["inv_cell"] = float(inv[0])
    out["ngas"] = int(ngas)
    return out


# ------------------------------------------------------------------ Morton
def morton_codes(pos, bits=21):
    pos = _f64(pos, (-1, 3))
    codes = np.empty(pos.shape[0], np.uint64)
    lib().orc_morton(_p(pos), pos.shape[0], bits, _p(codes), None, None)
    return codes


def morton_codes_numpy(pos, bits=21):
    """numpy restatement of core/solvers/barnes_hut.py:38-46 (same float64
    operation order; interleave by a bit loop)."""
    pos = _f64(pos, (-1, 3))
    lo = pos.min(axis=0)
    span = float((pos.max(axis=0) - lo).max())
    span = span if span > 0 else 1.0
    qmax = 2 ** bits - 1
    scale = qmax / (span * 1.0000001)
    q = np.clip((pos - lo) * scale, 0, qmax).astype(np.uint64)
    code = np.zeros(pos.shape[0], np.uint64)
    for b in range(bits):
        for k in range(3):
            code |= ((q[:, k] >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b + k)
    return code


def stable_argsort(codes):
    codes = np.ascontiguousarray(codes, dtype=np.uint64)
    order = np.empty(codes.size, np.int32)
    lib().orc_stable_argsort_u64(_p(codes), codes.size, _p(order))
    return order


# --------------------------------------------------------------- LBVH tree
def build_radix(sorted_codes):
    code = np.ascontiguousarray(sorted_codes).astype(np.int64)
    n = code.size
    left = np.zeros(max(n - 1, 1), np.int32)
    right = np.zeros(max(n - 1, 1), np.int32)
    parent = np.full(max(2 * n - 1, 1), -1, np.int32)
    lib().orc_build_radix(_p(code), n, _p(left), _p(right), _p(parent))
    return left, right, parent


def summaries(order, pos, mass, parent):
    order = np.ascontiguousarray(order, dtype=np.int32)
    pos = _f64(pos, (-1, 3))
    mass = _f64(mass, (-1,))
    parent = np.ascontiguousarray(parent, dtype=np.int32)
    n = pos.shape[0]
    m = max(2 * n - 1, 1)
    com = np.zeros((m, 3))
    nmass = np.zeros(m)
    nmin = np.zeros((m, 3))
    nmax = np.zeros((m, 3))
    lib().orc_summaries(_p(order), _p(pos), _p(mass), _p(parent), n, _p(com),
                        _p(nmass), _p(nmin), _p(nmax))
    return com, nmass, nmin, nmax


def traverse(pos, order, com, nmass, nmin, nmax, left, right, theta, eps2, G,
             max_stack=64, targets=None):
    """Returns (acc, dropped_pushes).  acc rows follow ``targets`` when given."""
    pos = _f64(pos, (-1, 3))
    n = pos.shape[0]
    args = [np.ascontiguousarray(order, dtype=np.int32), _f64(com, (-1, 3)),
            _f64(nmass, (-1,)), _f64(nmin, (-1, 3)), _f64(nmax, (-1, 3)),
            np.ascontiguousarray(left, dtype=np.int32),
            np.ascontiguousarray(right, dtype=np.int32)]
    if targets is None:
        t, nt = None, n
    else:
        t = np.ascontiguousarray(targets, dtype=np.int64)
        nt = t.size
    acc = np.zeros((nt, 3))
    dropped = lib().orc_traverse(_p(pos), *[_p(a) for a in args], n,
                                 float(theta) ** 2, eps2, max_stack, G,
                                 _p(t) if t is not None else None, nt, _p(acc))
    return acc, dropped


def traverse_phi(pos, order, com, nmass, nmin, nmax, left, right, theta, eps2,
                 max_stack=64, targets=None):
    """The tree potential of the same walk as ``traverse``: for each target
    sum m / sqrt(|d|^2 + eps2) over the accepted nodes and other leaves (no
    G).  Returns (phi, dropped_pushes)."""
    pos = _f64(pos, (-1, 3))
    n = pos.shape[0]
    args = [np.ascontiguousarray(order, dtype=np.int32), _f64(com, (-1, 3)),
            _f64(nmass, (-1,)), _f64(nmin, (-1, 3)), _f64(nmax, (-1, 3)),
            np.ascontiguousarray(left, dtype=np.int32),
            np.ascontiguousarray(right, dtype=np.int32)]
    if targets is None:
        t, nt = None, n
    else:
        t = np.ascontiguousarray(targets, dtype=np.int64)
        nt = t.size
    acc = np.zeros((nt, 3))
    phi = np.zeros(nt)
    dropped = lib().orc_traverse_phi(_p(pos), *[_p(a) for a in args], n,
                                     float(theta) ** 2, eps2, max_stack, 1.0,
                                     _p(t) if t is not None else None, nt,
                                     _p(acc), _p(phi))
    return phi, dropped


def group_walk(pos, tree, theta, eps2, G, group=32):
    """Accelerations and potentials (no G) of every particle from the group
    walk over ``tree`` (``bh_tree``'s dict): the maximal subtrees with at
    most ``group`` leaves share the node set their bounding box accepts.
    Returns (acc, phi) indexed by particle."""
    pos = _f64(pos, (-1, 3))
    n = pos.shape[0]
    acc = np.zeros((n, 3))
    phi = np.zeros(n)
    args = [np.ascontiguousarray(tree["order"], dtype=np.int32), _f64(tree["com"], (-1, 3)),
            _f64(tree["nmass"], (-1,)), _f64(tree["nmin"], (-1, 3)), _f64(tree["nmax"], (-1, 3)),
            np.ascontiguousarray(tree["left"], dtype=np.int32),
            np.ascontiguousarray(tree["right"], dtype=np.int32)]
    lib().orc_group_walk(_p(pos), *[_p(a) for a in args], n, group, float(theta) ** 2, eps2, G,
                         _p(acc), _p(phi))
    return acc, phi


def bh_tree(pos, mass, bits=21):
    """Stages 1-4 of BarnesHut.compute: keys, order, topology, summaries."""
    codes = morton_codes(pos, bits)
    order = stable_argsort(codes)
    left, right, parent = build_radix(codes[order])
    com, nmass, nmin, nmax = summaries(order, pos, mass, parent)
    return dict(code=codes, order=order, left=left, right=right,
                parent=parent, com=com, nmass=nmass, nmin=nmin, nmax=nmax)


def bh_compute(pos, mass, theta, softening, G, bits=21, max_stack=64,
               targets=None):
    """BarnesHut(n, theta, softening, max_stack).compute (with the key width
    as a parameter).  Returns (acc, tree, dropped)."""
    t = bh_tree(pos, mass, bits)
    acc, dropped = traverse(pos, t["order"], t["com"], t["nmass"], t["nmin"],
                            t["nmax"], t["left"], t["right"], theta,
                            float(softening) ** 2, G, max_stack, targets)
    return acc, t, dropped
