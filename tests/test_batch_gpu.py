"""Batched direct N^2 (many systems, one persistent launch per step) against
the single-system path and the FP64 oracle.

Tolerances: accelerations as in the direct tests (per-particle relative RMS
<= 1e-5, max <= 1e-5 against FP64); trajectories of the batched launch and
of the per-system loop differ only by FP32 summation order, so after a few
steps positions agree to 1e-5 of the system size.
"""
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG_NAME

pytestmark = pytest.mark.gpu


def _mods():
    return (importlib.import_module(PKG_NAME + ".batch"), importlib.import_module(PKG_NAME + ".ic"),
            importlib.import_module(PKG_NAME + ".autotune"))


def _systems(ic, sizes):
    out = []
    for s, n in enumerate(sizes):
        p, v, m = ic.plummer(n, seed=100 + s)
        f = lambda a: a.astype(np.float32).astype(np.float64)
        out.append((f(p), f(v), f(m)))
    return out


def _rel(a, ref):
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)


@pytest.mark.parametrize("tiles", [(2, 4), (2, 8), (4, 4), (4, 8)])
def test_batch_acc_matches_oracle(cuda_dev, orc, tiles):
    batch, ic, _ = _mods()
    sizes = [1, 2, 33, 256, 1000, 1025, 3000, 700, 4096, 17]
    systems = _systems(ic, sizes)
    b = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev, tiles=tiles)
    b.compute_acc()
    acc = b.a4[:, :3].double().cpu().numpy()
    for s, (p, v, m) in enumerate(systems):
        o0, o1 = b.offsets[s], b.offsets[s + 1]
        ref = orc.direct_acc(p, m, 1.0, 0.02 ** 2)
        if sizes[s] == 1:
            assert np.all(acc[o0:o1] == 0.0)
            continue
        rel = _rel(acc[o0:o1], ref)
        assert np.sqrt((rel ** 2).mean()) < 1e-5 and rel.max() < 1e-5, (s, rel.max())


@pytest.mark.parametrize("graph", [False, True])
def test_batch_kdk_matches_loop(cuda_dev, graph):
    batch, ic, _ = _mods()
    sizes = ic.batch_sizes(24, 256, 4096)
    systems = _systems(ic, sizes)
    b1 = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev)
    b2 = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev)
    b1.run(1e-3, 5, graph=graph)
    b1.run(1e-3, 5, graph=graph)  # graph replay with the same key
    b2.run_loop(1e-3, 10)
    torch.cuda.synchronize()
    x1 = b1.xm[:, :3].double().cpu().numpy()
    x2 = b2.xm[:, :3].double().cpu().numpy()
    assert np.abs(x1 - x2).max() < 1e-5 * np.abs(x2).max()
    v1 = b1.v4[:, :3].double().cpu().numpy()
    v2 = b2.v4[:, :3].double().cpu().numpy()
    assert np.abs(v1 - v2).max() < 1e-4 * np.abs(v2).max()
    assert b1.launch_count() == 2 * 10 + 2  # initial acc + 2 launches per step


def test_batch_matches_oracle_kdk(cuda_dev, orc):
    batch, ic, _ = _mods()
    systems = _systems(ic, [300, 1200, 64])
    b = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev)
    b.run(1e-3, 8)
    for s, (p, v, m) in enumerate(systems):
        a0 = orc.direct_acc(p, m, 1.0, 4e-4)
        pr, vr, _ = orc.kdk_direct(p, v, a0, m, 1.0, 4e-4, 1e-3, 8)
        gp, gv, _ = b.system(s)
        assert np.abs(gp - pr).max() < 2e-5 * np.abs(pr).max()
        assert np.abs(gv - vr).max() < 1e-4 * np.abs(vr).max()


def test_batch_energy_drift_and_autotune(cuda_dev):
    batch, ic, tune = _mods()
    grav = importlib.import_module(PKG_NAME + ".solvers.gravity")
    sizes = ic.batch_sizes(16, 256, 2048)
    systems = _systems(ic, sizes)
    b = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev)
    shape, times = tune.tune_batch(b, use_cache=False)
    assert shape in tune.BATCH_SHAPES and len(times) == len(tune.BATCH_SHAPES)
    g = grav.DirectGravity(int(max(sizes)), cuda_dev)

    def energies():
        out = []
        for s in range(len(sizes)):
            o0, o1 = int(b.offsets[s]), int(b.offsets[s + 1])
            out.append(g.energies(b.xm[o0:o1], b.v4[o0:o1], 1.0, 4e-4)[2])
        return np.array(out)

    e0 = energies()
    b.run(1e-3, 50)
    e1 = energies()
    assert np.abs((e1 - e0) / e0).max() < 1e-3


def test_batch_bad_arguments(cuda_dev):
    pkg = importlib.import_module(PKG_NAME)
    batch, ic, _ = _mods()
    b = batch.DirectBatch(_systems(ic, [10, 20]), device=cuda_dev)
    with pytest.raises(pkg.GravityError):
        b.set_tiles(3, 4)
    with pytest.raises(ValueError):
        batch.DirectBatch([], device=cuda_dev)


# ------------------------------------------------- symmetric batched pass
def test_batch_sym_acc_matches_oracle(cuda_dev, orc):
    batch, ic, _ = _mods()
    sizes = [1, 2, 33, 256, 1000, 1025, 3000, 700, 4096, 17, 512, 513]
    systems = _systems(ic, sizes)
    b = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev, variant=1)
    acc = b.a4[:, :3].double().cpu().numpy()
    assert torch.all(b.a4[:, 3] == 0.0)
    for s, (p, v, m) in enumerate(systems):
        o0, o1 = b.offsets[s], b.offsets[s + 1]
        if sizes[s] == 1:
            assert np.all(acc[o0:o1] == 0.0)
            continue
        rel = _rel(acc[o0:o1], orc.direct_acc(p, m, 1.0, 0.02 ** 2))
        assert np.sqrt((rel ** 2).mean()) < 1e-5 and rel.max() < 1e-5, (s, rel.max())
    b.close()


@pytest.mark.parametrize("graph", [False, True])
def test_batch_sym_kdk_matches_loop_and_repeats(cuda_dev, graph):
    batch, ic, _ = _mods()
    sizes = ic.batch_sizes(24, 256, 4096)
    systems = _systems(ic, sizes)
    b1 = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev, variant=1)
    b3 = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev, variant=1)
    b2 = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev)
    for b in (b1, b3):
        b.run(1e-3, 5, graph=graph)
        b.run(1e-3, 5, graph=graph)
    b2.run_loop(1e-3, 10)
    torch.cuda.synchronize()
    for t1, t3 in zip((b1.xm, b1.v4, b1.a4), (b3.xm, b3.v4, b3.a4)):
        assert torch.equal(t1, t3)
    x1 = b1.xm[:, :3].double().cpu().numpy()
    x2 = b2.xm[:, :3].double().cpu().numpy()
    assert np.abs(x1 - x2).max() < 1e-5 * np.abs(x2).max()
    v1 = b1.v4[:, :3].double().cpu().numpy()
    v2 = b2.v4[:, :3].double().cpu().numpy()
    assert np.abs(v1 - v2).max() < 1e-4 * np.abs(v2).max()
    assert b1.launch_count() == 2 * 10 + 2
    for b in (b1, b2, b3):
        b.close()


def test_batch_sym_graph_equals_direct_launches(cuda_dev):
    """Switching the variant recaptures the graph; replay and direct launches
    give the same bits."""
    batch, ic, _ = _mods()
    systems = _systems(ic, [900, 2500, 130])
    out = []
    for graph in (False, True):
        b = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev)
        b.run(1e-3, 2, graph=graph)
        b.set_variant(1)
        b.run(1e-3, 3, graph=graph)
        b.set_variant(0)
        b.run(1e-3, 2, graph=graph)
        torch.cuda.synchronize()
        out.append((b.xm.clone(), b.v4.clone(), b.a4.clone()))
        b.close()
    for u, w in zip(*out):
        assert torch.equal(u, w)


def test_batch_bad_variant(cuda_dev):
    batch, ic, _ = _mods()
    pkg = importlib.import_module(PKG_NAME)
    b = batch.DirectBatch(_systems(ic, [64, 65]), device=cuda_dev)
    with pytest.raises(pkg.GravityError):
        b.set_variant(2)
    b.close()


def test_batch_sym_scratch_limit_is_an_error_and_autotune_skips_it(cuda_dev):
    """One 400k-particle system needs about 5 GB of tile-pair slots: selecting
    the symmetric batch pass fails cleanly and the per-target pass stays."""
    batch, ic, tune = _mods()
    pkg = importlib.import_module(PKG_NAME)
    p, v, m = ic.plummer(400_000, seed=5)
    b = batch.DirectBatch([(p, v, m)], G=1.0, softening=0.02, device=cuda_dev)
    with pytest.raises(pkg.GravityError):
        b.set_variant(1)
    b.run(1e-3, 1, graph=False)  # still the per-target pass
    torch.cuda.synchronize()
    assert torch.isfinite(b.xm).all()
    shape, times = tune.tune_batch(b, reps=1, use_cache=False)
    assert shape[2] == 0 and "2,4,1" not in times
    b.close()


def test_batch_sym_one_slice_matches_oracle(cuda_dev, orc):
    """40 systems of 16,384 particles: enough tile pairs (21,120) for one
    source slice per pair; accelerations of three systems on sampled
    targets against the oracle."""
    batch, ic, _ = _mods()
    systems = _systems(ic, [16384] * 40)
    b = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev, variant=1)
    acc = b.a4[:, :3].double().cpu().numpy()
    rng = np.random.default_rng(3)
    for s in (0, 17, 39):
        p, v, m = systems[s]
        o0 = b.offsets[s]
        t = rng.choice(16384, 512, replace=False)
        rel = _rel(acc[o0 + t], orc.direct_acc(p, m, 1.0, 0.02 ** 2, t))
        assert np.sqrt((rel ** 2).mean()) < 1e-5 and rel.max() < 1e-5, (s, rel.max())
    b.close()


@pytest.mark.parametrize("variant", [0, 1])
def test_config4_batch_512_systems(cuda_dev, orc, variant):
    """The batching workload at full size: 512 Plummer spheres with N
    log-uniform in [256, 16384] (seed s), eps = 0.02, one persistent launch
    for all of them.  Four seeded targets per system (2,048 in all) against
    the FP64 oracle of their own system, RMS and max <= 1e-5; then one KDK
    step of the whole batch against the oracle's step on four systems."""
    batch, ic, _ = _mods()
    systems = [(_f(p), _f(v), _f(m)) for p, v, m in ic.plummer_batch(512)]
    b = batch.DirectBatch(systems, G=1.0, softening=0.02, device=cuda_dev, variant=variant)
    acc = b.a4[:, :3].double().cpu().numpy()
    rng = np.random.default_rng(5)
    got, ref = [], []
    for s, (p, v, m) in enumerate(systems):
        t = rng.choice(p.shape[0], 4, replace=False)
        got.append(acc[b.offsets[s] + t])
        ref.append(orc.direct_acc(p, m, 1.0, 4e-4, t))
    rel = _rel(np.vstack(got), np.vstack(ref))
    assert np.sqrt((rel ** 2).mean()) < 1e-5 and rel.max() < 1e-5, rel.max()
    b.run(1e-3, 1)
    for s in (0, 17, 255, 511):
        p, v, m = systems[s]
        a0 = orc.direct_acc(p, m, 1.0, 4e-4)
        pr, vr, _ = orc.kdk_direct(p, v, a0, m, 1.0, 4e-4, 1e-3, 1)
        gp, gv, _ = b.system(s)
        assert np.abs(gp - pr).max() < 1e-6 * np.abs(pr).max()
        assert np.abs(gv - vr).max() < 1e-5 * np.abs(vr).max()
    b.close()


def _f(a):
    return a.astype(np.float32).astype(np.float64)
