"""Tile-shape autotuner for the direct-sum kernels.

Times every candidate shape (targets per lane k, warps per CTA, inner-loop
variant) on the caller's actual workload with CUDA events and keeps the
fastest.  Results are cached per GPU and workload signature in
_build/autotune.json next to the library, so later runs reuse them.
"""
from __future__ import annotations

import json
import os
import time

import torch

from . import _buildlib
from ._lib import GravityError

CACHE = os.path.join(_buildlib.BUILD, "autotune.json")
# (k, warps, variant); the symmetric variant 2 has one tile shape of its own.
DIRECT_SHAPES = [(k, w, packed) for k in (2, 4) for w in (4, 8) for packed in (0, 1)] + [(2, 4, 2)]
# (k, warps, variant); variant 1 is the symmetric batched pass (one shape).
BATCH_SHAPES = [(k, w, 0) for k in (2, 4) for w in (4, 8)] + [(2, 4, 1)]


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except Exception:
        return {}


def _save(d):
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + f".tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def _time(fn, reps: int) -> float:
    fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def _key(kind: str, sig) -> str:
    return f"{torch.cuda.get_device_name()}|{kind}|{sig}"


def tune_direct(solver, xm, G=1.0, eps2=1e-4, reps=3, use_cache=True):
    """Pick (k, warps, packed) for DirectGravity `solver` on positions `xm`;
    sets it on the solver and returns (shape, {shape: ms})."""
    n = xm.shape[0]
    bucket = 1 << max(0, (n - 1).bit_length())
    key = _key("direct", bucket)
    cache = _load() if use_cache else {}
    if key in cache and len(cache[key]["best"]) == 3:
        shape = tuple(cache[key]["best"])
        solver.set_tiles(shape[0], shape[1], 0, shape[2])
        return shape, cache[key]["ms"]
    acc = torch.zeros_like(xm)
    times = {}
    for k, w, packed in DIRECT_SHAPES:
        solver.set_tiles(k, w, 0, packed)
        times[f"{k},{w},{packed}"] = _time(lambda: solver.acc(xm, acc, G, eps2), reps)
    best = min(times, key=times.get)
    shape = tuple(int(x) for x in best.split(","))
    solver.set_tiles(shape[0], shape[1], 0, shape[2])
    cache = _load()
    cache[key] = {"best": list(shape), "ms": times, "when": time.time()}
    _save(cache)
    return shape, times


def tune_batch(batch, dt=1e-3, reps=2, use_cache=True):
    """Pick (k, warps, variant) for a DirectBatch by timing one KDK step per
    candidate on a copy of its state (the batch is restored afterwards)."""
    sig = f"{batch.n_total}:{len(batch.sizes)}:{int(batch.sizes.max())}:{batch.interactions_per_step()}"
    key = _key("batch", sig)
    cache = _load() if use_cache else {}
    if key in cache and len(cache[key]["best"]) == 3:
        k, w, v = cache[key]["best"]
        batch.set_tiles(k, w)
        batch.set_variant(v)
        return (k, w, v), cache[key]["ms"]
    saved = batch.state_arrays()
    times = {}
    for k, w, v in BATCH_SHAPES:
        batch.set_tiles(k, w)
        try:
            batch.set_variant(v)
        except GravityError:  # the symmetric pass's scratch would be too large
            continue
        times[f"{k},{w},{v}"] = _time(lambda: batch.run(dt, 1, graph=False), reps)
        batch.restore(saved)
    best = min(times, key=times.get)
    k, w, v = (int(x) for x in best.split(","))
    batch.set_tiles(k, w)
    batch.set_variant(v)
    cache = _load()
    cache[key] = {"best": [k, w, v], "ms": times, "when": time.time()}
    _save(cache)
    return (k, w, v), times
