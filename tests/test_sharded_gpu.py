"""Target slices of the direct sum on the GPU (gb_direct_acc_range) and the
sharded KDK stepper on one rank.

The slices a W-rank run computes are computed here one after the other on
one GPU (no kernel waits on another): every slice against the FP64 oracle
(max relative error <= 1e-5, the direct path's bound), and the slices put
together against the whole-system call (same terms, another stream-K split:
within FP32 rounding of the compensated sums).
"""
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG_NAME

pytestmark = pytest.mark.gpu

MAX_TOL = 1e-5


def _mods():
    grav = importlib.import_module(PKG_NAME + ".solvers.gravity")
    ic = importlib.import_module(PKG_NAME + ".ic")
    sh = importlib.import_module(PKG_NAME + ".sharded")
    lib = importlib.import_module(PKG_NAME + "._lib")
    return grav, ic, sh, lib


def _f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def _rel(a, ref):
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)


@pytest.mark.parametrize("n,world", [(20000, 2), (20000, 3), (5000, 8), (1000, 3), (300, 4)])
@pytest.mark.parametrize("variant", [0, 1, 2])
def test_slices_match_oracle_and_whole_call(cuda_dev, orc, n, world, variant):
    grav, ic, sh, _ = _mods()
    pos, _, mass = ic.plummer(n, seed=11)
    pos, mass = _f32(pos), _f32(mass)
    xm = torch.tensor(np.column_stack((pos, mass)), dtype=torch.float32, device=cuda_dev)
    g = grav.DirectGravity(n, cuda_dev)
    g.set_variant(variant)
    whole = torch.zeros_like(xm)
    g.acc(xm, whole, 1.0, 1e-4)
    acc = torch.zeros_like(xm)
    phi = torch.zeros(n, device=cuda_dev)
    for r in range(world):
        t0, nt, _ = sh.shard_range(n, r, world)
        a_r = torch.full((max(nt, 1), 4), 7.0, device=cuda_dev)  # overwritten, not added to
        p_r = torch.zeros(max(nt, 1), device=cuda_dev)
        g.acc_range(xm, n, t0, nt, a_r, 1.0, 1e-4, phi=p_r)
        acc[t0:t0 + nt] = a_r[:nt]
        phi[t0:t0 + nt] = p_r[:nt]
    torch.cuda.synchronize()
    a = acc[:, :3].double().cpu().numpy()
    sample = np.random.default_rng(n).choice(n, min(n, 2048), replace=False)
    ref = orc.direct_acc(pos, mass, 1.0, 1e-4, sample)
    assert _rel(a[sample], ref).max() < MAX_TOL
    assert _rel(a, whole[:, :3].double().cpu().numpy()).max() < 5e-6
    ref_phi = orc.phi_targets(pos, mass, 1e-4, sample)
    got_phi = phi.double().cpu().numpy()[sample]
    assert (np.abs(got_phi - ref_phi) / np.abs(ref_phi)).max() < MAX_TOL
    g.close()


def test_range_flags_and_errors(cuda_dev, orc):
    grav, ic, _, lib = _mods()
    n = 3000
    pos, _, mass = ic.plummer(n, seed=2)
    pos, mass = _f32(pos), _f32(mass)
    xm = torch.tensor(np.column_stack((pos, mass)), dtype=torch.float32, device=cuda_dev)
    g = grav.DirectGravity(n, cuda_dev)
    base = torch.ones((1000, 4), device=cuda_dev)
    acc = base.clone()
    g.acc_range(xm, n, 1000, 1000, acc, 1.0, 1e-4, accumulate=True)
    fresh = torch.zeros_like(base)
    g.acc_range(xm, n, 1000, 1000, fresh, 1.0, 1e-4)
    plain = torch.zeros_like(base)
    g.acc_range(xm, n, 1000, 1000, plain, 1.0, 1e-4, plain=True)
    torch.cuda.synchronize()
    ref = orc.direct_acc(pos, mass, 1.0, 1e-4, np.arange(1000, 2000))
    assert _rel(fresh[:, :3].double().cpu().numpy(), ref).max() < MAX_TOL
    # GB_ACCUMULATE adds the same sums to what acc held (one FP32 add).
    assert torch.equal(acc[:, :3], base[:, :3] + fresh[:, :3])
    assert _rel(plain[:, :3].double().cpu().numpy(), ref).max() < 1e-4  # plain FP32 sums
    for t0, nt in ((-1, 10), (2990, 11), (0, n + 1)):
        with pytest.raises(lib.GravityError) as e:
            g.acc_range(xm, n, t0, nt, torch.zeros((max(nt, 1), 4), device=cuda_dev), 1.0, 1e-4)
        assert e.value.status == lib.GB_EINVAL
    with pytest.raises(lib.GravityError) as e:
        lib.call("gb_direct_acc_range", g.handle, xm.data_ptr(), n, 0, 10, acc.data_ptr(), None, 1.0, 1e-4,
                 lib.GB_USE_GRAPH, None)
    assert e.value.status == lib.GB_EINVAL
    g.close()


def test_sharded_stepper_one_rank_matches_oracle(cuda_dev, orc):
    """ShardedDirect on one rank (CUDA ops): the split KDK loop with the
    range force pass against the oracle's KDK loop; energies against the
    oracle's sums."""
    _, ic, sh, _ = _mods()
    n, steps, dt = 4000, 5, 1e-3
    pos, vel, mass = ic.plummer(n, seed=4)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    s = sh.ShardedDirect(pos, vel, mass, G=1.0, softening=0.01, device=cuda_dev)
    s.run(dt, steps)
    p, v, _ = s.gather_state()
    acc0 = orc.direct_acc(pos, mass, 1.0, 1e-4)
    pr, vr, _ = orc.kdk_direct(pos, vel, acc0, mass, 1.0, 1e-4, dt, steps)
    assert np.abs(p - pr).max() < 1e-5 * np.abs(pr).max()
    assert np.abs(v - vr).max() < 1e-4 * np.abs(vr).max()
    ke, pe, tot = s.energies()
    ke_ref = orc.kinetic_energy(v, mass)
    pe_ref = orc.potential_energy(p, mass, 1.0, 1e-4)
    assert abs(ke - ke_ref) < 1e-5 * abs(ke_ref) and abs(pe - pe_ref) < 1e-5 * abs(pe_ref)
    s.close()


# ------------------------------------------------------------------- tree
@pytest.mark.parametrize("tpl", [-1, 0, 1, 2, 3])
def test_tree_slices_equal_whole_traversal(cuda_dev, tpl):
    """gb_bh_accel_range over the key-order slices of 3 ranks, each into a
    zeroed array, summed: equal to one gb_bh_accel (and its potentials) bit
    for bit in every traversal shape; slices that are not warp-aligned
    included."""
    _, ic, sh, lib = _mods()
    bhmod = importlib.import_module(PKG_NAME + ".solvers.barnes_hut")
    n = 30001
    pos, _, mass = ic.exponential_disk(n, seed=21)
    xm = torch.tensor(np.column_stack((pos, mass)), dtype=torch.float32, device=cuda_dev)
    b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, key_bits=10, device=cuda_dev)
    b.set_traversal(tpl)
    b.build(xm)
    whole = torch.zeros_like(xm)
    phi_whole = torch.zeros(n, device=cuda_dev)
    b.accel(whole, phi=phi_whole)
    total = torch.zeros_like(xm)
    phi_total = torch.zeros(n, device=cuda_dev)
    for r in range(3):
        s0, ns, _ = sh.shard_range(n, r, 3)
        part = torch.zeros_like(xm)
        phi_part = torch.zeros(n, device=cuda_dev)
        b.accel_range(part, s0, ns, phi=phi_part)
        total += part
        phi_total += phi_part
    torch.cuda.synchronize()
    assert torch.equal(total, whole) and torch.equal(phi_total, phi_whole)
    with pytest.raises(lib.GravityError) as e:
        b.accel_range(total, n - 5, 10)
    assert e.value.status == lib.GB_EINVAL
    b.close()


def test_tree_sharded_stepper_one_rank_equals_fused_kdk(cuda_dev):
    """ShardedBarnesHut on one rank (kick, drift, replicated build, the
    range traversal over all targets, kick) follows gb_bh_kdk's fused step
    bit for bit; its energies equal the tree handle's."""
    _, ic, sh, _ = _mods()
    bhmod = importlib.import_module(PKG_NAME + ".solvers.barnes_hut")
    n, steps, dt = 20000, 4, 1e-4
    pos, vel, mass = ic.exponential_disk(n, seed=22)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    s = sh.ShardedBarnesHut(pos, vel, mass, theta=0.5, softening=0.05, key_bits=10, device=cuda_dev)
    s.run(dt, steps)
    p, v, a = s.gather_state()
    b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, key_bits=10, device=cuda_dev)
    xm = torch.tensor(np.column_stack((pos, mass)), dtype=torch.float32, device=cuda_dev)
    v4 = torch.zeros_like(xm)
    v4[:, :3] = torch.tensor(vel, dtype=torch.float32, device=cuda_dev)
    a4 = torch.zeros_like(xm)
    b.compute(xm, a4)
    phi = torch.zeros(n, device=cuda_dev)
    b.kdk(xm, v4, a4, dt, steps, phi=phi)
    assert np.array_equal(p, xm[:, :3].double().cpu().numpy())
    assert np.array_equal(v, v4[:, :3].double().cpu().numpy())
    assert np.array_equal(a, a4[:, :3].double().cpu().numpy())
    e = s.energies()
    e_ref = b.energies_from_phi(xm, v4, phi)
    assert e == e_ref
    s.close()
    b.close()
