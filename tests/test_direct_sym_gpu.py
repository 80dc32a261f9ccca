"""Symmetric direct-sum pass (gb_direct_set_variant 2: each unordered pair
once, applied to both particles) against the FP64 oracle.

Same tolerances as the per-target pass (per-particle relative error, RMS
<= 1e-5, max <= 1e-5); the fused KDK form is checked against the oracle's
leapfrog and, bit for bit, against itself under CUDA-graph replay.
"""
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG_NAME

pytestmark = pytest.mark.gpu

RMS_TOL = 1e-5
MAX_TOL = 1e-5
SYM = 2


def _mods():
    grav = importlib.import_module(PKG_NAME + ".solvers.gravity")
    ic = importlib.import_module(PKG_NAME + ".ic")
    return grav, ic


def _f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def _xm(pos, mass, dev):
    return torch.tensor(np.column_stack((pos, mass)), dtype=torch.float32, device=dev)


def _rel(a, ref):
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)


def _sym_solver(grav, n, dev):
    s = grav.DirectGravity(n, dev)
    s.set_tiles(2, 4, 0, SYM)
    return s


@pytest.mark.parametrize("plain", [False, True])
def test_plummer_20k_matches_oracle(cuda_dev, orc, plain):
    grav, ic = _mods()
    pos, _, mass = ic.plummer(20000, seed=0)
    pos, mass = _f32(pos), _f32(mass)
    xm = _xm(pos, mass, cuda_dev)
    s = _sym_solver(grav, 20000, cuda_dev)
    acc = torch.zeros_like(xm)
    s.acc(xm, acc, 1.0, 1e-4, plain=plain)
    a = acc[:, :3].double().cpu().numpy()
    targets = np.random.default_rng(1).choice(20000, 2048, replace=False)
    ref = orc.direct_acc(pos, mass, 1.0, 1e-4, targets)
    rel = _rel(a[targets], ref)
    assert np.sqrt((rel ** 2).mean()) < RMS_TOL, np.sqrt((rel ** 2).mean())
    assert rel.max() < MAX_TOL, rel.max()
    s.close()


@pytest.mark.parametrize("n", [1, 2, 3, 33, 511, 512, 513, 1025, 4099, 9000])
def test_ragged_sizes(cuda_dev, orc, n):
    """Ragged last tiles and one tile (all with 4 source slices per tile
    pair)."""
    grav, ic = _mods()
    pos, _, mass = ic.plummer(max(n, 2), seed=n)
    pos, mass = _f32(pos[:n]), _f32(mass[:n])
    xm = _xm(pos, mass, cuda_dev)
    s = _sym_solver(grav, n, cuda_dev)
    acc = torch.full_like(xm, 7.0)
    s.acc(xm, acc, 2.5, 0.05 ** 2)
    a = acc[:, :3].double().cpu().numpy()
    assert torch.all(acc[:, 3] == 0.0)
    if n == 1:
        assert np.all(a == 0.0)
        return
    ref = orc.direct_acc(pos, mass, 2.5, 0.05 ** 2)
    assert _rel(a, ref).max() < MAX_TOL
    s.close()


@pytest.mark.parametrize("n", [70001, 90001, 110001])
def test_fewer_source_slices_match_oracle(cuda_dev, orc, n):
    """4, 2 and 1 source slices per tile pair at N = 70,001, 90,001 and
    110,001 on a 152-SM GB300 (the slice count falls as the tile pairs
    outnumber 16x the resident CTAs), on 2,048 sampled targets."""
    grav, ic = _mods()
    pos, _, mass = ic.plummer(n, seed=41)
    pos, mass = _f32(pos), _f32(mass)
    xm = _xm(pos, mass, cuda_dev)
    s = _sym_solver(grav, n, cuda_dev)
    acc = torch.zeros_like(xm)
    s.acc(xm, acc, 1.0, 1e-4)
    targets = np.random.default_rng(2).choice(n, 2048, replace=False)
    rel = _rel(acc[:, :3].double().cpu().numpy()[targets], orc.direct_acc(pos, mass, 1.0, 1e-4, targets))
    assert np.sqrt((rel ** 2).mean()) < RMS_TOL and rel.max() < MAX_TOL, rel.max()
    s.close()


def test_matches_per_target_pass_and_is_deterministic(cuda_dev):
    grav, ic = _mods()
    pos, _, mass = ic.plummer(30000, seed=3)
    xm = _xm(pos, mass, cuda_dev)
    s = _sym_solver(grav, 30000, cuda_dev)
    a1, a2, a3 = (torch.zeros_like(xm) for _ in range(3))
    s.acc(xm, a1, 1.0, 1e-4)
    s.acc(xm, a2, 1.0, 1e-4)
    s.set_tiles(2, 4, 0, 0)
    s.acc(xm, a3, 1.0, 1e-4)
    torch.cuda.synchronize()
    assert torch.equal(a1, a2)
    rel = _rel(a1[:, :3].double().cpu().numpy(), a3[:, :3].double().cpu().numpy())
    assert np.sqrt((rel ** 2).mean()) < RMS_TOL and rel.max() < MAX_TOL, rel.max()
    s.close()


def test_accumulate_and_potential(cuda_dev, orc):
    grav, ic = _mods()
    ext = importlib.import_module(PKG_NAME + ".solvers.external")
    pos, _, mass = ic.plummer(3000, seed=4)
    pos, mass = _f32(pos), _f32(mass)
    xm = _xm(pos, mass, cuda_dev)
    s = _sym_solver(grav, 3000, cuda_dev)
    acc = torch.zeros_like(xm)
    acc[:, 0] = 1.0
    s.acc(xm, acc, 1.0, 1e-4, accumulate=True)
    a = acc[:, :3].double().cpu().numpy()
    ref = orc.direct_acc(pos, mass, 1.0, 1e-4)
    ref[:, 0] += 1.0
    assert _rel(a, ref).max() < MAX_TOL
    p = {"M_d": 5.0, "a": 3.0, "b": 0.3, "M_h": 50.0, "a_h": 20.0, "smbh_mass": 0.1, "is_hernquist": True}
    pot = ext.Potential.from_dict(p)
    base = np.zeros((3000, 3))
    acc2 = torch.zeros_like(xm)
    ext.direct_acc_ext(s, xm, acc2, 1.0, 1e-4, pot, accumulate=False)
    got = acc2[:, :3].double().cpu().numpy()
    ref2 = orc.grav_ext_acc(pos, mass, 1.0, 1e-4, p, base)
    assert _rel(got, ref2).max() < MAX_TOL
    s.close()


def test_kdk_matches_oracle_and_graph_replay(cuda_dev, orc):
    grav, ic = _mods()
    pos, vel, mass = ic.plummer(2048, seed=6)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    out = []
    for graph in (False, True):
        xm = _xm(pos, mass, cuda_dev)
        v4 = torch.zeros_like(xm)
        v4[:, :3] = torch.tensor(vel, dtype=torch.float32, device=cuda_dev)
        a4 = torch.zeros_like(xm)
        s = _sym_solver(grav, 2048, cuda_dev)
        s.acc(xm, a4, 1.0, 1e-4)
        s.kdk(xm, v4, a4, 1.0, 1e-4, 1e-3, 6, graph=graph)
        s.kdk(xm, v4, a4, 1.0, 1e-4, 1e-3, 4, graph=graph)
        torch.cuda.synchronize()
        out.append((xm.clone(), v4.clone(), a4.clone()))
        s.close()
    for u, w in zip(*out):
        assert torch.equal(u, w)
    a0 = orc.direct_acc(pos, mass, 1.0, 1e-4)
    p, v, _ = orc.kdk_direct(pos, vel, a0, mass, 1.0, 1e-4, 1e-3, 10)
    xm, v4, _ = out[0]
    assert np.abs(xm[:, :3].double().cpu().numpy() - p).max() < 2e-5 * np.abs(p).max()
    assert np.abs(v4[:, :3].double().cpu().numpy() - v).max() < 1e-4 * np.abs(v).max()


def test_variant_out_of_range_is_rejected(cuda_dev):
    pkg = importlib.import_module(PKG_NAME)
    grav, _ = _mods()
    s = grav.DirectGravity(64, cuda_dev)
    with pytest.raises(pkg.GravityError):
        s.set_tiles(2, 4, 0, 3)
    s.close()


def test_kdk_graph_recaptures_after_scratch_regrowth(cuda_dev):
    """The symmetric force pass and the symmetric adjoint share the handle's
    tile-pair scratch.  An adjoint step on a larger system regrows it; the
    next graph-replayed KDK step must capture again (the scratch address is
    part of the graph key) and match direct launches bit for bit."""
    grav, ic = _mods()
    lib = importlib.import_module(PKG_NAME + "._lib")
    n_small, n_big = 1000, 4096
    p, v, m = ic.plummer(n_small, seed=21)
    pb, _, mb = ic.plummer(n_big, seed=22)
    stream = torch.cuda.current_stream(cuda_dev).cuda_stream
    out = []
    for graph in (False, True):
        s = _sym_solver(grav, n_big, cuda_dev)
        xm = _xm(p, m, cuda_dev)
        v4 = torch.zeros_like(xm)
        v4[:, :3] = torch.tensor(v, dtype=torch.float32, device=cuda_dev)
        a4 = torch.zeros_like(xm)
        s.acc(xm, a4, 1.0, 1e-4)
        s.kdk(xm, v4, a4, 1.0, 1e-4, 1e-3, 3, graph=graph)
        xb = _xm(pb, mb, cuda_dev)
        lx, lv, la = (torch.ones_like(xb) for _ in range(3))
        lm = torch.zeros(n_big, dtype=torch.float32, device=cuda_dev)
        lib.call("gb_adjoint_set_variant", s.handle, 2)
        lib.call("gb_adjoint_step", s.handle, xb.data_ptr(), lx.data_ptr(), lv.data_ptr(), la.data_ptr(),
                 lm.data_ptr(), n_big, 1.0, 1e-4, 1e-3, 0, stream)
        s.kdk(xm, v4, a4, 1.0, 1e-4, 1e-3, 3, graph=graph)
        torch.cuda.synchronize()
        out.append((xm.clone(), v4.clone(), a4.clone(), lx.clone(), lm.clone()))
        s.close()
    for u, w in zip(*out):
        assert torch.equal(u, w)


BAND_5_PAIRS = 5 * 16 * 512 * 5  # slot bytes for 5 tile pairs with 4 source slices


def test_bands_match_oracle_and_single_pass(cuda_dev, orc):
    """A small band budget splits N = 5,000 into 9 bands of tile rows; the
    result matches the oracle and the one-band pass up to rounding order."""
    grav, ic = _mods()
    n = 5000
    pos, _, mass = ic.plummer(n, seed=31)
    pos, mass = _f32(pos), _f32(mass)
    xm = _xm(pos, mass, cuda_dev)
    s1 = _sym_solver(grav, n, cuda_dev)
    s2 = _sym_solver(grav, n, cuda_dev)
    s2.set_sym_band(BAND_5_PAIRS)
    a1, a2, a3 = (torch.zeros_like(xm) for _ in range(3))
    s1.acc(xm, a1, 1.0, 1e-4)
    s2.acc(xm, a2, 1.0, 1e-4)
    s2.acc(xm, a3, 1.0, 1e-4)
    torch.cuda.synchronize()
    assert torch.equal(a2, a3)
    assert s2.launch_count() > s1.launch_count()
    ref = orc.direct_acc(pos, mass, 1.0, 1e-4)
    rel = _rel(a2[:, :3].double().cpu().numpy(), ref)
    assert np.sqrt((rel ** 2).mean()) < RMS_TOL and rel.max() < MAX_TOL, rel.max()
    rel12 = _rel(a2[:, :3].double().cpu().numpy(), a1[:, :3].double().cpu().numpy())
    assert rel12.max() < 1e-5
    # acc += form in bands
    a4 = torch.zeros_like(xm)
    a4[:, 1] = 2.0
    s2.acc(xm, a4, 1.0, 1e-4, accumulate=True)
    ref[:, 1] += 2.0
    assert _rel(a4[:, :3].double().cpu().numpy(), ref).max() < MAX_TOL
    s1.close()
    s2.close()


def test_bands_kdk_graph_and_oracle(cuda_dev, orc):
    grav, ic = _mods()
    n = 3000
    pos, vel, mass = ic.plummer(n, seed=32)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    out = []
    for graph in (False, True):
        xm = _xm(pos, mass, cuda_dev)
        v4 = torch.zeros_like(xm)
        v4[:, :3] = torch.tensor(vel, dtype=torch.float32, device=cuda_dev)
        a4 = torch.zeros_like(xm)
        s = _sym_solver(grav, n, cuda_dev)
        s.set_sym_band(BAND_5_PAIRS)
        s.acc(xm, a4, 1.0, 1e-4)
        s.kdk(xm, v4, a4, 1.0, 1e-4, 1e-3, 4, graph=graph)
        s.set_sym_band(1 << 30)  # one band from here: the graph is captured again
        s.kdk(xm, v4, a4, 1.0, 1e-4, 1e-3, 2, graph=graph)
        torch.cuda.synchronize()
        out.append((xm.clone(), v4.clone(), a4.clone()))
        s.close()
    for u, w in zip(*out):
        assert torch.equal(u, w)
    a0 = orc.direct_acc(pos, mass, 1.0, 1e-4)
    p, v, _ = orc.kdk_direct(pos, vel, a0, mass, 1.0, 1e-4, 1e-3, 6)
    xm, v4, _ = out[0]
    assert np.abs(xm[:, :3].double().cpu().numpy() - p).max() < 2e-5 * np.abs(p).max()
    assert np.abs(v4[:, :3].double().cpu().numpy() - v).max() < 1e-4 * np.abs(v).max()


def test_band_budget_validation(cuda_dev):
    pkg = importlib.import_module(PKG_NAME)
    grav, _ = _mods()
    s = grav.DirectGravity(64, cuda_dev)
    with pytest.raises(pkg.GravityError):
        s.set_sym_band(1000)
    s.close()


@pytest.fixture(scope="module")
def merger(orc):
    """The precision workload: two unit Plummer spheres of 131,072 particles
    (G = 1) 10 apart on a parabolic orbit, eps = 0.01, and the FP64 oracle's
    accelerations of 8,192 seeded targets."""
    grav, ic = _mods()
    pos, _, mass = ic.plummer_pair(131072)
    pos, mass = _f32(pos), _f32(mass)
    targets = np.random.default_rng(0).choice(pos.shape[0], 8192, replace=False)
    return pos, mass, targets, orc.direct_acc(pos, mass, 1.0, 1e-4, targets)


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_config3_merger_full_size(cuda_dev, merger, variant):
    """Every force-pass form on the full 2 x 131,072 merger against FP64 on
    8,192 targets: RMS and max <= 1e-5 (the symmetric pass runs in two bands
    of tile rows at this size, with running sums between them)."""
    grav, _ = _mods()
    pos, mass, targets, ref = merger
    xm = _xm(pos, mass, cuda_dev)
    s = grav.DirectGravity(pos.shape[0], cuda_dev)
    s.set_variant(variant)
    acc = torch.zeros_like(xm)
    s.acc(xm, acc, 1.0, 1e-4)
    torch.cuda.synchronize()
    rel = _rel(acc[:, :3].double().cpu().numpy()[targets], ref)
    assert np.sqrt((rel ** 2).mean()) < RMS_TOL, np.sqrt((rel ** 2).mean())
    assert rel.max() < MAX_TOL, rel.max()
    s.close()
