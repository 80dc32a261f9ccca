"""Analytic galaxy potential (Miyamoto-Nagai disk, Hernquist or Plummer halo,
central point mass) on the device against the reference's own outputs
(tests/golden/analytic.npz from grav_analytic / add_analytic / add_grav_ext)
and the FP64 oracle.

Tolerances: the potential is evaluated in FP32 from FP32 positions, so the
acceleration a call adds agrees with the FP64 reference to a relative 1e-5
per particle (plus 1e-6 of the largest term, for particles where the terms
cancel); direct self-gravity as in the direct tests (per-particle relative
RMS <= 1e-5 of the FP64 sum).  Fused and separate passes differ only by the
FP32 rounding of one extra addition.
"""
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG_NAME, load_golden

pytestmark = pytest.mark.gpu

NAMES = ["mn_plummer", "hernquist_smbh", "mn_hernquist_smbh"]


def _mods():
    return (importlib.import_module(PKG_NAME + ".solvers.external"),
            importlib.import_module(PKG_NAME + ".solvers.gravity"),
            importlib.import_module(PKG_NAME + ".solvers.barnes_hut"),
            importlib.import_module(PKG_NAME))


def _pot_dict(g, name):
    return {k: g[f"{name}_{k}"].item() for k in ("M_d", "a", "b", "M_h", "a_h", "is_hernquist", "smbh_mass")}


def _xm(pos, mass, dev):
    xm = torch.zeros((pos.shape[0], 4), dtype=torch.float32, device=dev)
    xm[:, :3] = torch.tensor(pos, dtype=torch.float32, device=dev)
    xm[:, 3] = torch.tensor(mass, dtype=torch.float32, device=dev)
    return xm


def _acc4(acc3, dev):
    a = torch.zeros((acc3.shape[0], 4), dtype=torch.float32, device=dev)
    a[:, :3] = torch.tensor(acc3, dtype=torch.float32, device=dev)
    return a


def _check_increment(got, base, ref):
    """got - base against ref - base, per particle."""
    inc = got - base
    inc_ref = ref - base
    scale = np.abs(inc_ref).max()
    err = np.linalg.norm(inc - inc_ref, axis=1)
    bound = 1e-5 * np.linalg.norm(inc_ref, axis=1) + 1e-6 * scale
    assert np.all(np.isfinite(got))
    assert np.all(err <= bound), (err / np.maximum(bound, 1e-300)).max()


@pytest.mark.parametrize("name", NAMES)
def test_analytic_acc_matches_reference(cuda_dev, name):
    ext, _, _, _ = _mods()
    g = load_golden("analytic")
    pot = ext.Potential.from_dict(_pot_dict(g, name))
    xm = _xm(g["pos"], g["mass"], cuda_dev)
    acc = _acc4(g["acc0"], cuda_dev)
    ext.analytic_acc(xm, acc, pot, float(g["G"]), accumulate=True)
    got = acc[:, :3].double().cpu().numpy()
    base = g["acc0"].astype(np.float32).astype(np.float64)
    _check_increment(got, base, g[f"{name}_grav_analytic"])
    # Without GB_ACCUMULATE the call writes the analytic term alone.
    acc2 = torch.full_like(acc, 7.0)
    ext.analytic_acc(xm, acc2, pot, float(g["G"]), accumulate=False)
    _check_increment(acc2[:, :3].double().cpu().numpy(), np.zeros_like(base),
                     g[f"{name}_grav_analytic"] - g["acc0"])


@pytest.mark.parametrize("name", NAMES)
def test_reference_named_mirrors(cuda_dev, name):
    """grav_analytic / add_grav_ext called with the reference's argument
    lists."""
    ext, _, _, _ = _mods()
    g = load_golden("analytic")
    p = _pot_dict(g, name)
    args = (p["M_d"], p["a"], p["b"], p["M_h"], p["a_h"], p["is_hernquist"], p["smbh_mass"])
    n = g["pos"].shape[0]
    xm = _xm(g["pos"], g["mass"], cuda_dev)
    base = g["acc0"].astype(np.float32).astype(np.float64)
    acc = _acc4(g["acc0"], cuda_dev)
    ext.grav_analytic(xm, acc, n, *args, G=float(g["G"]))
    _check_increment(acc[:, :3].double().cpu().numpy(), base, g[f"{name}_grav_analytic"])
    acc = _acc4(g["acc0"], cuda_dev)
    ext.add_grav_ext(xm, acc, n, float(g["eps2"]), *args, G=float(g["G"]))
    got = acc[:, :3].double().cpu().numpy()
    inc, inc_ref = got - base, g[f"{name}_add_grav_ext"] - base
    rel = np.linalg.norm(inc - inc_ref, axis=1) / np.linalg.norm(inc_ref, axis=1)
    assert np.sqrt((rel ** 2).mean()) < 1e-5 and rel.max() < 1e-4, rel.max()


@pytest.mark.parametrize("accumulate", [True, False])
def test_direct_acc_ext_fused_matches_oracle(cuda_dev, orc, accumulate):
    ext, grav, _, _ = _mods()
    g = load_golden("analytic")
    G, eps2 = float(g["G"]), float(g["eps2"])
    p = _pot_dict(g, "mn_hernquist_smbh")
    pot = ext.Potential.from_dict(p)
    n = g["pos"].shape[0]
    xm = _xm(g["pos"], g["mass"], cuda_dev)
    solver = grav.DirectGravity(n, cuda_dev)
    base = g["acc0"].astype(np.float32).astype(np.float64) if accumulate else np.zeros((n, 3))
    acc = _acc4(base, cuda_dev)
    ext.direct_acc_ext(solver, xm, acc, G, eps2, pot, accumulate=accumulate)
    got = acc[:, :3].double().cpu().numpy()
    ref = orc.grav_ext_acc(g["pos"], g["mass"], G, eps2, p, base)
    inc, inc_ref = got - base, ref - base
    rel = np.linalg.norm(inc - inc_ref, axis=1) / np.linalg.norm(inc_ref, axis=1)
    assert np.sqrt((rel ** 2).mean()) < 1e-5 and rel.max() < 1e-4, rel.max()
    # Fused against separate passes: gb_direct_acc then gb_analytic_acc.
    acc2 = _acc4(base, cuda_dev)
    solver.acc(xm, acc2, G, eps2, accumulate=accumulate)
    ext.analytic_acc(xm, acc2, pot, G, accumulate=True)
    sep = acc2[:, :3].double().cpu().numpy()
    np.testing.assert_allclose(got, sep, rtol=2e-6, atol=2e-6 * np.abs(sep).max())
    solver.close()


def test_null_potential_is_the_plain_call(cuda_dev):
    """pot = NULL gives exactly gb_direct_acc / gb_bh_accel."""
    ext, grav, bhm, _ = _mods()
    ic = importlib.import_module(PKG_NAME + ".ic")
    pos, _, mass = ic.exponential_disk(5000, seed=3)
    xm = _xm(pos, mass, cuda_dev)
    solver = grav.DirectGravity(5000, cuda_dev)
    a1 = torch.zeros_like(xm)
    a2 = torch.zeros_like(xm)
    solver.acc(xm, a1, 43009.1725, 0.0025)
    ext.direct_acc_ext(solver, xm, a2, 43009.1725, 0.0025, None, accumulate=False)
    assert torch.equal(a1, a2)
    bh = bhm.BarnesHut(5000, theta=0.5, softening=0.05, device=cuda_dev)
    b1 = torch.zeros_like(xm)
    b2 = torch.zeros_like(xm)
    bh.compute(xm, b1)
    ext.tree_forces_ext(bh, xm, b2, None, accumulate=False)
    assert torch.equal(b1, b2)
    solver.close()
    bh.close()


@pytest.mark.parametrize("name", NAMES)
def test_tree_forces_ext_matches_separate_passes_and_oracle(cuda_dev, orc, name):
    """Tree forces + potential in one traversal against the tree forces and
    gb_analytic_acc as two passes, and against the FP64 oracle (tree
    traversal + analytic terms)."""
    ext, _, bhm, _ = _mods()
    ic = importlib.import_module(PKG_NAME + ".ic")
    g = load_golden("analytic")
    p = _pot_dict(g, name)
    pot = ext.Potential.from_dict(p)
    n = 6000
    pos, _, mass = ic.exponential_disk(n, seed=9)
    pos = pos.astype(np.float32).astype(np.float64)
    mass = mass.astype(np.float32).astype(np.float64)
    G, theta, soft = 43009.1725, 0.5, 0.05
    xm = _xm(pos, mass, cuda_dev)
    base = np.random.default_rng(1).normal(0.0, 1e3, (n, 3)).astype(np.float32).astype(np.float64)
    bh = bhm.BarnesHut(n, theta=theta, softening=soft, G=G, device=cuda_dev)
    fused = _acc4(base, cuda_dev)
    ext.tree_forces_ext(bh, xm, fused, pot, accumulate=True)
    sep = _acc4(base, cuda_dev)
    bh.compute(xm, sep, accumulate=True)
    ext.analytic_acc(xm, sep, pot, G, accumulate=True)
    f = fused[:, :3].double().cpu().numpy()
    s = sep[:, :3].double().cpu().numpy()
    np.testing.assert_allclose(f, s, rtol=2e-6, atol=2e-6 * np.abs(s).max())
    tree, _, _ = orc.bh_compute(pos, mass, theta, soft, G, bits=21)
    ref = orc.analytic_acc(pos, G, p, base + tree)
    inc, inc_ref = f - base, ref - base
    rel = np.linalg.norm(inc - inc_ref, axis=1) / np.linalg.norm(inc_ref, axis=1)
    assert np.sqrt((rel ** 2).mean()) < 1e-5 and rel.max() < 1e-3, (np.sqrt((rel ** 2).mean()), rel.max())
    bh.close()


def test_bad_potential_is_rejected(cuda_dev):
    ext, grav, _, pkg = _mods()
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    import ctypes
    xm = torch.zeros((16, 4), dtype=torch.float32, device=cuda_dev)
    acc = torch.zeros_like(xm)
    for bad in (lib_mod.Potential(5.0, 3.0, 0.3, 12.0, 8.0, 0.0, 2, 0),
                lib_mod.Potential(float("nan"), 3.0, 0.3, 12.0, 8.0, 0.0, 0, 0),
                lib_mod.Potential(5.0, 3.0, 0.3, 12.0, 8.0, 0.0, 0, 1)):
        with pytest.raises(pkg.GravityError):
            lib_mod.call("gb_analytic_acc", xm.data_ptr(), acc.data_ptr(), 16, 1.0, ctypes.addressof(bad), 0,
                         torch.cuda.current_stream().cuda_stream)
    with pytest.raises(pkg.GravityError):
        lib_mod.call("gb_analytic_acc", xm.data_ptr(), acc.data_ptr(), 16, 1.0, None, 0,
                     torch.cuda.current_stream().cuda_stream)
