"""gb_direct_acc_noalloc: the direct force sum for callers that cannot
allocate device memory (their own memory pool owns the GPU, they run inside
another framework's arena, or they must never block on cudaMalloc/cudaFree).

Called through the C ABI and compared, on the same inputs, with the
allocating entry point gb_direct_acc and with the FP64 oracle on seeded
targets.  The calls run back to back, so each one reuses the static scratch
the previous one left behind.  The sizes cover both launch plans (source
units of 128 and of 32 particles) and a single-CTA system; the flags
GB_ACCUMULATE and GB_PLAIN_FP32 are covered too.  Tolerance of the other
direct-sum tests: per-particle relative difference RMS <= 1e-5, max <= 1e-5.
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG_NAME

pytestmark = pytest.mark.gpu

RMS_TOL = 1e-5
MAX_TOL = 1e-5


def _rel(a, ref):
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)


def _check(a, ref, what):
    rel = _rel(a, ref)
    assert np.all(np.isfinite(a)), what
    assert np.sqrt((rel ** 2).mean()) < RMS_TOL, (what, np.sqrt((rel ** 2).mean()))
    assert rel.max() < MAX_TOL, (what, rel.max())


def _mods():
    pkg = importlib.import_module(PKG_NAME)
    pkg.load_library()
    return (pkg, importlib.import_module(PKG_NAME + "._lib"),
            importlib.import_module(PKG_NAME + ".solvers.gravity"),
            importlib.import_module(PKG_NAME + ".ic"))


def _noalloc(lib_mod, dev, xm, acc, G, eps2, flags=0):
    lib_mod.call("gb_direct_acc_noalloc", xm.data_ptr(), acc.data_ptr(), xm.shape[0], float(G),
                 float(eps2), flags, torch.cuda.current_stream(dev).cuda_stream)


def _system(ic, n, seed, dev):
    pos, _, mass = ic.plummer(max(n, 2), seed=seed)
    pos = pos[:n].astype(np.float32).astype(np.float64)
    mass = mass[:n].astype(np.float32).astype(np.float64)
    xm = torch.tensor(np.column_stack((pos, mass)), dtype=torch.float32, device=dev)
    return pos, mass, xm


# (n, seed, G, eps): 65,536 and 20,000 take 128-source units, 10,000 takes
# 32-source units, 100 runs on one CTA.
CASES = [(65536, 1, 1.0, 0.01), (10000, 2, 2.5, 0.05), (100, 3, 1.0, 0.02), (20000, 4, 1.0, 0.01)]


def test_noalloc_matches_allocating_call_and_oracle(cuda_dev, orc):
    _, lib_mod, grav, ic = _mods()
    for call, (n, seed, G, eps) in enumerate(CASES):
        pos, mass, xm = _system(ic, n, seed, cuda_dev)
        ref = torch.zeros_like(xm)
        grav.DirectGravity(n, cuda_dev).acc(xm, ref, G, eps * eps)
        out = torch.full_like(xm, float("nan")) if call % 2 == 0 else torch.zeros_like(xm)
        _noalloc(lib_mod, cuda_dev, xm, out, G, eps * eps)
        torch.cuda.synchronize()
        a = out[:, :3].double().cpu().numpy()
        _check(a, ref[:, :3].double().cpu().numpy(), ("vs gb_direct_acc", n))
        targets = np.random.default_rng(seed).choice(n, min(n, 2048), replace=False)
        _check(a[targets], orc.direct_acc(pos, mass, G, eps * eps, targets), ("vs oracle", n))


def test_noalloc_flags(cuda_dev, orc):
    _, lib_mod, _, ic = _mods()
    n = 10000
    pos, mass, xm = _system(ic, n, 7, cuda_dev)
    targets = np.random.default_rng(7).choice(n, 2048, replace=False)
    ref = orc.direct_acc(pos, mass, 1.0, 1e-4, targets)
    # GB_ACCUMULATE adds into a pre-filled acc.
    base = torch.zeros_like(xm)
    base[:, 0] = 3.0
    base[:, 2] = -1.5
    acc = base.clone()
    _noalloc(lib_mod, cuda_dev, xm, acc, 1.0, 1e-4, lib_mod.GB_ACCUMULATE)
    torch.cuda.synchronize()
    got = acc[:, :3].double().cpu().numpy()[targets]
    _check(got, ref + base[:, :3].double().cpu().numpy()[targets], "GB_ACCUMULATE")
    # GB_PLAIN_FP32: plain FP32 sums, still within the bound at this size.
    acc = torch.zeros_like(xm)
    _noalloc(lib_mod, cuda_dev, xm, acc, 1.0, 1e-4, lib_mod.GB_PLAIN_FP32)
    torch.cuda.synchronize()
    _check(acc[:, :3].double().cpu().numpy()[targets], ref, "GB_PLAIN_FP32")


def test_noalloc_rejects_what_it_cannot_do(cuda_dev):
    pkg, lib_mod, _, _ = _mods()
    big = torch.zeros((65536 + 1, 4), dtype=torch.float32, device=cuda_dev)
    with pytest.raises(pkg.GravityError, match="outside"):
        _noalloc(lib_mod, cuda_dev, big, big.clone(), 1.0, 1e-4)
    small = torch.zeros((16, 4), dtype=torch.float32, device=cuda_dev)
    with pytest.raises(pkg.GravityError, match="flags"):
        _noalloc(lib_mod, cuda_dev, small, small.clone(), 1.0, 1e-4, lib_mod.GB_USE_GRAPH)
