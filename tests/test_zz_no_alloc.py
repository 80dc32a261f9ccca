"""gb_direct_acc_noalloc: the direct force sum for callers that cannot
allocate device memory (their own memory pool owns the GPU, they run inside
another framework's arena, or they must never block on cudaMalloc/cudaFree).

Called through the C ABI and compared with the allocating entry point
gb_direct_acc on the same inputs, twice in a row (the second call reuses the
static scratch the first one left behind), with the tolerance of the other
direct-sum tests: per-particle relative difference RMS <= 1e-5, max <= 1e-4.
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
MAX_TOL = 1e-4


def _rel(a, ref):
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)


def _noalloc(lib_mod, dev, xm, acc, G, eps2, flags=0):
    lib_mod.call("gb_direct_acc_noalloc", xm.data_ptr(), acc.data_ptr(), xm.shape[0], float(G),
                 float(eps2), flags, torch.cuda.current_stream(dev).cuda_stream)


def test_noalloc_matches_allocating_call_twice(cuda_dev):
    pkg = importlib.import_module(PKG_NAME)
    pkg.load_library()
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    grav = importlib.import_module(PKG_NAME + ".solvers.gravity")
    ic = importlib.import_module(PKG_NAME + ".ic")
    nmax = 65536
    for call, (n, seed, G, eps) in enumerate([(65536, 1, 1.0, 0.01), (20000, 2, 2.5, 0.05)]):
        pos, _, mass = ic.plummer(n, seed=seed)
        xm = torch.tensor(np.column_stack((pos, mass)), dtype=torch.float32, device=cuda_dev)
        ref = torch.zeros_like(xm)
        grav.DirectGravity(n, cuda_dev).acc(xm, ref, G, eps * eps)
        out = torch.full_like(xm, float("nan")) if call == 0 else torch.zeros_like(xm)
        _noalloc(lib_mod, cuda_dev, xm, out, G, eps * eps)
        torch.cuda.synchronize()
        a = out[:, :3].double().cpu().numpy()
        r = ref[:, :3].double().cpu().numpy()
        rel = _rel(a, r)
        assert np.all(np.isfinite(a))
        assert np.sqrt((rel ** 2).mean()) < RMS_TOL, (call, np.sqrt((rel ** 2).mean()))
        assert rel.max() < MAX_TOL, (call, rel.max())
    # Sizes beyond the static scratch are refused, nothing is launched.
    big = torch.zeros((nmax + 1, 4), dtype=torch.float32, device=cuda_dev)
    with pytest.raises(pkg.GravityError, match="outside"):
        _noalloc(lib_mod, cuda_dev, big, big.clone(), 1.0, 1e-4)
