"""The potential as an epilogue of the force pass (direct and tree), against
the FP64 oracle.

Direct: phi_i = sum_{j != i} m_j / sqrt(|d|^2 + eps^2) of potential_energy
(core/solvers/gravity.py:47-55), written by the force pass itself; every
force-pass form, against the oracle on seeded targets with the direct-sum
tolerance (per-particle relative error RMS and max <= 1e-5).  The forces of
a pass that also writes phi are bit-identical to the plain pass's.

Tree: the monopole potential of the nodes the traversal accepts, checked
against the oracle's FP64 walk over the same node set with the tolerance of
the tree forces (median <= 1e-5, 99th percentile <= 1e-4, max <= 1e-2: a
node whose acceptance test sits on the FP32/FP64 rounding boundary can
flip), and against the FP64 direct sum within the monopole budget at
theta = 0.5 (median <= 5e-3, max <= 1.5e-2; the FP64 walk itself is at
3.5e-3 / 7.4e-3 on a disk).
"""
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG_NAME

pytestmark = pytest.mark.gpu


def _mods():
    return (importlib.import_module(PKG_NAME), importlib.import_module(PKG_NAME + ".solvers.gravity"),
            importlib.import_module(PKG_NAME + ".solvers.barnes_hut"), importlib.import_module(PKG_NAME + ".ic"))


def _f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def _xm(pos, mass, dev):
    return torch.tensor(np.column_stack((pos, mass)), dtype=torch.float32, device=dev)


def _rel_scalar(a, ref):
    return np.abs(a - ref) / np.maximum(np.abs(ref), 1e-300)


def _check_direct(phi, ref):
    rel = _rel_scalar(phi, ref)
    assert np.sqrt((rel ** 2).mean()) < 1e-5, np.sqrt((rel ** 2).mean())
    assert rel.max() < 1e-5, rel.max()


def _check_tree(phi, ref):
    rel = _rel_scalar(phi, ref)
    assert np.median(rel) < 1e-5, np.median(rel)
    assert np.percentile(rel, 99) < 1e-4, np.percentile(rel, 99)
    assert rel.max() < 1e-2, rel.max()


@pytest.mark.parametrize("variant,band", [(0, None), (1, None), (2, None), (2, 1 << 22)])
@pytest.mark.parametrize("plain", [False, True])
def test_direct_acc_phi(cuda_dev, orc, variant, band, plain):
    """Every force-pass form (the symmetric one also in many bands of tile
    rows, with running potential sums between them)."""
    _, grav, _, ic = _mods()
    n = 20000
    pos, _, mass = ic.plummer(n, seed=3)
    pos, mass = _f32(pos), _f32(mass)
    xm = _xm(pos, mass, cuda_dev)
    s = grav.DirectGravity(n, cuda_dev)
    s.set_variant(variant)
    if band is not None:
        s.set_sym_band(band)
    a_plain = torch.zeros_like(xm)
    s.acc(xm, a_plain, 1.0, 1e-4, plain=plain)
    acc = torch.zeros_like(xm)
    phi = torch.full((n,), float("nan"), device=cuda_dev)
    s.acc_phi(xm, acc, phi, 1.0, 1e-4, plain=plain)
    torch.cuda.synchronize()
    assert torch.equal(acc, a_plain)
    targets = np.random.default_rng(4).choice(n, 2048, replace=False)
    _check_direct(phi.double().cpu().numpy()[targets], orc.phi_targets(pos, mass, 1e-4, targets))
    s.close()


@pytest.mark.parametrize("n", [1, 2, 33, 4099])
def test_direct_acc_phi_ragged(cuda_dev, orc, n):
    _, grav, _, ic = _mods()
    pos, _, mass = ic.plummer(max(n, 2), seed=n)
    pos, mass = _f32(pos[:n]), _f32(mass[:n])
    xm = _xm(pos, mass, cuda_dev)
    for variant in (0, 2):
        s = grav.DirectGravity(n, cuda_dev)
        s.set_variant(variant)
        acc = torch.zeros_like(xm)
        phi = torch.full((n,), float("nan"), device=cuda_dev)
        s.acc_phi(xm, acc, phi, 1.0, 0.05 ** 2)
        torch.cuda.synchronize()
        got = phi.double().cpu().numpy()
        if n == 1:
            assert got[0] == 0.0
        else:
            _check_direct(got, orc.phi_targets(pos, mass, 0.05 ** 2, np.arange(n)))
        s.close()


@pytest.mark.parametrize("variant", [0, 2])
@pytest.mark.parametrize("graph", [False, True])
def test_direct_kdk_phi(cuda_dev, orc, variant, graph):
    """11 KDK steps whose last step also writes phi: the state equals 11
    plain steps bit for bit, and phi is the potential of the final
    positions."""
    _, grav, _, ic = _mods()
    n = 6000
    pos, vel, mass = ic.plummer(n, seed=9)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    out = []
    for with_phi in (False, True):
        s = grav.DirectGravity(n, cuda_dev)
        s.set_variant(variant)
        xm = _xm(pos, mass, cuda_dev)
        v4 = torch.zeros_like(xm)
        v4[:, :3] = torch.tensor(vel, dtype=torch.float32, device=cuda_dev)
        a4 = torch.zeros_like(xm)
        s.acc(xm, a4, 1.0, 1e-4)
        phi = torch.full((n,), float("nan"), device=cuda_dev) if with_phi else None
        s.kdk(xm, v4, a4, 1.0, 1e-4, 1e-3, 11, graph=graph, phi=phi)
        s.kdk(xm, v4, a4, 1.0, 1e-4, 1e-3, 3, graph=graph, phi=phi)  # graph slots reused
        torch.cuda.synchronize()
        out.append((xm.clone(), v4.clone(), a4.clone(), phi))
        s.close()
    for u, w in zip(out[0][:3], out[1][:3]):
        assert torch.equal(u, w)
    xm, phi = out[1][0], out[1][3]
    p1 = xm[:, :3].double().cpu().numpy()
    targets = np.random.default_rng(2).choice(n, 1024, replace=False)
    _check_direct(phi.double().cpu().numpy()[targets], orc.phi_targets(p1, mass, 1e-4, targets))


def test_energy_from_phi(cuda_dev, orc):
    _, grav, _, ic = _mods()
    n = 8000
    pos, vel, mass = ic.plummer(n, seed=5)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    xm = _xm(pos, mass, cuda_dev)
    v4 = torch.zeros_like(xm)
    v4[:, :3] = torch.tensor(vel, dtype=torch.float32, device=cuda_dev)
    s = grav.DirectGravity(n, cuda_dev)
    s.set_variant(2)
    phi = torch.zeros(n, device=cuda_dev)
    s.acc_phi(xm, torch.zeros_like(xm), phi, 1.0, 1e-4)
    e_phi = s.energies_from_phi(xm, v4, phi, 1.0)
    e_ref = (orc.kinetic_energy(vel, mass), orc.potential_energy(pos, mass, 1.0, 1e-4))
    assert abs(e_phi[0] - e_ref[0]) < 1e-6 * abs(e_ref[0])
    assert abs(e_phi[1] - e_ref[1]) < 1e-6 * abs(e_ref[1])
    assert abs(e_phi[2] - (e_phi[0] + e_phi[1])) < 1e-12 * abs(e_phi[1])


def _bh_case(ic, n, seed):
    pos, vel, mass = ic.exponential_disk(n, seed=seed)
    return _f32(pos), _f32(vel), _f32(mass)


@pytest.mark.parametrize("tpl", [-1, 0, 1, 2])
def test_bh_accel_phi(cuda_dev, orc, tpl):
    """Tree potential of every traversal shape: forces bit-identical to the
    plain traversal, phi against the FP64 walk and the FP64 direct sum."""
    _, _, bhmod, ic = _mods()
    n = 50000
    pos, _, mass = _bh_case(ic, n, 14)
    b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, key_bits=10, device=cuda_dev)
    b.set_traversal(tpl)
    xm = _xm(pos, mass, cuda_dev)
    a_plain = torch.zeros_like(xm)
    b.compute(xm, a_plain)
    acc = torch.zeros_like(xm)
    phi = torch.full((n,), float("nan"), device=cuda_dev)
    b.compute(xm, acc, phi=phi)
    torch.cuda.synchronize()
    assert torch.equal(acc, a_plain)
    got = phi.double().cpu().numpy()
    assert np.all(np.isfinite(got)) and np.all(got > 0)
    t = orc.bh_tree(pos, mass, bits=10)
    targets = np.random.default_rng(3).choice(n, 4096, replace=False)
    ref_tree, _ = orc.traverse_phi(pos, t["order"], t["com"], t["nmass"], t["nmin"], t["nmax"], t["left"],
                                   t["right"], 0.5, 0.0025, targets=targets)
    _check_tree(got[targets], ref_tree)
    rel = _rel_scalar(got[targets], orc.phi_targets(pos, mass, 0.0025, targets))
    assert np.median(rel) < 5e-3 and rel.max() < 1.5e-2, (np.median(rel), rel.max())
    b.close()


@pytest.mark.parametrize("graph", [True, False])
def test_bh_kdk_phi(cuda_dev, graph):
    """KDK steps whose last step writes the tree potential: the state equals
    the plain steps' bit for bit, and phi equals that of a fresh build on
    the final positions."""
    _, _, bhmod, ic = _mods()
    n = 30000
    pos, vel, mass = _bh_case(ic, n, 15)
    out = []
    for with_phi in (False, True):
        b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, key_bits=10, device=cuda_dev)
        b.set_graph(graph)
        xm = _xm(pos, mass, cuda_dev)
        v4 = torch.zeros_like(xm)
        v4[:, :3] = torch.tensor(vel, dtype=torch.float32, device=cuda_dev)
        a4 = torch.zeros_like(xm)
        b.compute(xm, a4)
        phi = torch.full((n,), float("nan"), device=cuda_dev) if with_phi else None
        b.kdk(xm, v4, a4, 1e-4, 4, phi=phi)
        b.kdk(xm, v4, a4, 1e-4, 2, phi=phi)
        torch.cuda.synchronize()
        out.append((xm.clone(), v4.clone(), a4.clone(), phi, b))
    for u, w in zip(out[0][:3], out[1][:3]):
        assert torch.equal(u, w)
    xm, phi, b = out[1][0], out[1][3], out[1][4]
    phi2 = torch.zeros_like(phi)
    b.compute(xm, torch.zeros_like(xm), phi=phi2)
    torch.cuda.synchronize()
    assert torch.equal(phi, phi2)


def test_bh_phi_1m_disk(cuda_dev, orc):
    """The 1M disk workload (theta 0.5, 30-bit keys): tree potential against
    the FP64 walk and the FP64 direct sum on 4,096 seeded targets."""
    _, _, bhmod, ic = _mods()
    n = 1_000_000
    pos, _, mass = _bh_case(ic, n, 0)
    b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, key_bits=10, device=cuda_dev)
    xm = _xm(pos, mass, cuda_dev)
    phi = torch.zeros(n, device=cuda_dev)
    b.compute(xm, torch.zeros_like(xm), phi=phi)
    got = phi.double().cpu().numpy()
    t = orc.bh_tree(pos, mass, bits=10)
    targets = np.random.default_rng(0).choice(n, 4096, replace=False)
    ref_tree, _ = orc.traverse_phi(pos, t["order"], t["com"], t["nmass"], t["nmin"], t["nmax"], t["left"],
                                   t["right"], 0.5, 0.0025, targets=targets)
    _check_tree(got[targets], ref_tree)
    rel = _rel_scalar(got[targets], orc.phi_targets(pos, mass, 0.0025, targets))
    assert np.median(rel) < 5e-3 and rel.max() < 1.5e-2, (np.median(rel), rel.max())
    b.close()


@pytest.mark.parametrize("mode", ["direct", "bh"])
def test_engine_energies_after_a_step(cuda_dev, orc, mode):
    """Engine.energies() right after step()/run() takes the potential the
    last force pass wrote: the direct mode's equals the exact pair sum (FP32
    Kahan vs FP64: 1e-6), the tree mode's is within the monopole budget of
    it; without fused_potential the values are the same; writing positions
    through the field view makes the Engine recompute."""
    pkg, _, _, ic = _mods()
    if mode == "direct":
        pos, vel, mass = ic.plummer(4000, seed=6)
        kw = dict(softening=0.01, G=1.0)
        tol = 1e-6
    else:
        pos, vel, mass = ic.exponential_disk(20000, seed=6)
        kw = dict(theta=0.5, softening=0.05, key_bits=10)
        tol = 5e-3
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    res = {}
    for fused in (True, False):
        eng = pkg.Engine(gravity_mode=mode, fused_potential=fused, device=cuda_dev, **kw)
        eng.load_state(pkg.State.from_arrays(pos, vel, mass))
        e0 = eng.energies()
        eng.step(1e-4 if mode == "bh" else 1e-3)
        eng.run(1e-4 if mode == "bh" else 1e-3, 5)
        e1 = eng.energies()
        ex = eng.energies(exact=True)
        st = eng.to_state()
        pe_ref = orc.potential_energy(st.pos, st.mass, eng.G, eng.eps2)
        ke_ref = orc.kinetic_energy(st.vel, st.mass)
        assert abs(e1[0] - ke_ref) < 1e-6 * abs(ke_ref)
        assert abs(e1[1] - pe_ref) < tol * abs(pe_ref), (e1[1], pe_ref)
        assert abs(ex[1] - pe_ref) < 1e-6 * abs(pe_ref)
        res[fused] = (e0, e1)
        # A write through the field view invalidates the stored potential.
        p2 = st.pos * 1.01
        eng.pos.from_numpy(p2)
        pe2 = orc.potential_energy(_f32(p2), st.mass, eng.G, eng.eps2)
        assert abs(eng.energies()[1] - pe2) < tol * abs(pe2)
    for a, b in zip(res[True], res[False]):
        np.testing.assert_allclose(a, b, rtol=1e-6)


@pytest.mark.parametrize("mode", ["direct", "bh"])
def test_engine_auto_potential_follows_the_print_cadence(cuda_dev, mode):
    """fused_potential="auto" (the default): a run loop that calls energies()
    every 5 steps pays a potential pass of its own for the first two calls
    only; from the third on, the step that ends at the predicted call writes
    the potential.  Trajectories equal the always-fused Engine's bit for bit
    and the energies agree with it (the fused and the separate potential
    differ by FP32 rounding order)."""
    pkg, _, _, ic = _mods()
    if mode == "direct":
        pos, vel, mass = ic.plummer(3000, seed=8)
        kw = dict(softening=0.01, G=1.0)
        dt = 1e-3
    else:
        pos, vel, mass = ic.exponential_disk(20000, seed=8)
        kw = dict(theta=0.5, softening=0.05, key_bits=10)
        dt = 1e-4
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    out = {}
    for fused in ("auto", True):
        eng = pkg.Engine(gravity_mode=mode, fused_potential=fused, device=cuda_dev, **kw)
        eng.load_state(pkg.State.from_arrays(pos, vel, mass))
        es = []
        for k in range(1, 31):
            eng.step(dt)
            if k % 5 == 0:
                es.append(eng.energies())
        out[fused] = (np.array(es), eng.to_state(), eng.potential_passes)
    assert out["auto"][2] == 2 and out[True][2] == 0
    np.testing.assert_array_equal(out["auto"][1].pos, out[True][1].pos)
    np.testing.assert_array_equal(out["auto"][1].vel, out[True][1].vel)
    np.testing.assert_allclose(out["auto"][0], out[True][0], rtol=2e-6 if mode == "direct" else 1e-5)
