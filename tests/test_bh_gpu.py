"""LBVH Barnes-Hut CUDA path against the reference fixtures and the oracle.

Bit-exact: Morton keys, sort permutation, Karras topology (left, right,
parent), node AABBs.  Node masses and centres of mass are FP32 on the device
(the reference sums in FP64): masses within 5e-6 relative, centres within
1e-5 of the system size.  Accelerations: the device
traversal is FP32, so per-particle relative differences from the FP64
traversal are ~1e-6; a node whose acceptance test sits on the FP32/FP64
rounding boundary can flip, which moves that particle by about one node's
multipole error.  Hence: median <= 1e-5, 99th percentile <= 1e-4, max <=
1e-2 against the FP64 traversal, and the BH error against direct N^2 must
match the FP64 traversal's own error within 1e-4.
"""
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG_NAME, load_golden

pytestmark = pytest.mark.gpu


def _mods():
    pkg = importlib.import_module(PKG_NAME)
    bh = importlib.import_module(PKG_NAME + ".solvers.barnes_hut")
    ic = importlib.import_module(PKG_NAME + ".ic")
    grav = importlib.import_module(PKG_NAME + ".solvers.gravity")
    return pkg, bh, ic, grav


def _f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def _xm(pos, mass, dev):
    return torch.tensor(np.column_stack((pos, mass)), dtype=torch.float32, device=dev)


def _rel(a, ref):
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)


def _check_acc(a, ref):
    rel = _rel(a, ref)
    assert np.median(rel) < 1e-5, np.median(rel)
    assert np.percentile(rel, 99) < 1e-4, np.percentile(rel, 99)
    assert rel.max() < 1e-2, rel.max()


def _run(bhmod, pos, mass, dev, theta=0.5, soft=0.05, bits=21, G=None, max_stack=64, tpl=2):
    kw = {} if G is None else {"G": G}
    n = pos.shape[0]
    b = bhmod.BarnesHut(n, theta=theta, softening=soft, max_stack=max_stack, key_bits=bits,
                        device=dev, **kw)
    b.set_traversal(tpl)
    xm = _xm(pos, mass, dev)
    acc = torch.zeros_like(xm)
    b.compute(xm, acc)
    torch.cuda.synchronize()
    return b, acc[:, :3].double().cpu().numpy()


@pytest.mark.parametrize("bits", [21, 10])
@pytest.mark.parametrize("tpl", [-1, 0, 1, 2])
def test_golden_tree_bit_exact(cuda_dev, bits, tpl):
    _, bhmod, _, _ = _mods()
    g = load_golden("bh")
    pre = f"b{bits}_"
    b, a = _run(bhmod, g["pos"], g["mass"], cuda_dev, bits=bits, G=float(g["G"]), tpl=tpl)
    t = b.tree_arrays()
    ref_sorted = g[pre + "code"][g[pre + "order"]]
    np.testing.assert_array_equal(t["code"], ref_sorted)
    np.testing.assert_array_equal(t["order"], g[pre + "order"])
    np.testing.assert_array_equal(t["left"], g[pre + "left"])
    np.testing.assert_array_equal(t["right"], g[pre + "right"])
    np.testing.assert_array_equal(t["parent"], g[pre + "parent"])
    np.testing.assert_array_equal(t["nmin"], g[pre + "nmin"])
    np.testing.assert_array_equal(t["nmax"], g[pre + "nmax"])
    np.testing.assert_allclose(t["nmass"], g[pre + "nmass"], rtol=5e-6)
    scale = np.abs(g["pos"]).max()
    np.testing.assert_allclose(t["com"], g[pre + "com"], rtol=0, atol=1e-5 * scale)
    _check_acc(a, g[pre + "acc"])
    assert b.diag()["stack_drops"] == 0


def test_golden_compute_and_duplicates(cuda_dev):
    _, bhmod, _, _ = _mods()
    g = load_golden("bh")
    _, a = _run(bhmod, g["pos"], g["mass"], cuda_dev, bits=21, G=float(g["G"]))
    _check_acc(a, g["compute_acc"])
    b, a = _run(bhmod, g["dup_pos"], g["dup_mass"], cuda_dev, theta=0.7, bits=10, G=float(g["G"]))
    t = b.tree_arrays()
    np.testing.assert_array_equal(t["order"], g["dup_order"])
    np.testing.assert_array_equal(t["left"], g["dup_left"])
    np.testing.assert_array_equal(t["right"], g["dup_right"])
    np.testing.assert_array_equal(t["parent"], g["dup_parent"])
    _check_acc(a, g["dup_acc"])


@pytest.mark.parametrize("tpl", [0, 1, 2])
def test_stack_rule_matches_reference(cuda_dev, orc, tpl):
    """max_stack=6 silently drops subtrees in the reference (:212); the
    device applies the same rule per lane and counts the drops."""
    _, bhmod, _, _ = _mods()
    g = load_golden("bh")
    pos, mass = g["pos"][:400], g["mass"][:400]
    b, a = _run(bhmod, pos, mass, cuda_dev, bits=21, G=float(g["G"]), max_stack=6, tpl=tpl)
    _check_acc(a, g["stk6_acc"])
    _, _, dropped = orc.bh_compute(pos, mass, 0.5, 0.05, float(g["G"]), max_stack=6)
    d = b.diag()["stack_drops"]
    assert dropped > 0 and abs(d - dropped) <= max(2, dropped // 100), (d, dropped)


def test_engine_bh_golden(cuda_dev):
    pkg, _, _, _ = _mods()
    g = load_golden("engine_bh")
    eng = pkg.Engine(softening=float(g["softening"]), gravity_mode="bh",
                     theta=float(g["theta"]), device=cuda_dev)
    eng.load_state(pkg.State.from_arrays(g["pos0"], g["vel0"], g["mass"]))
    assert eng._bh is not None
    _check_acc(eng.acc.to_numpy(), g["acc0"])
    for _ in range(int(g["nsteps"])):
        eng.step(float(g["dt"]))
    st = eng.to_state()
    assert np.abs(st.pos - g["pos"]).max() < 1e-5 * np.abs(g["pos"]).max()
    assert np.abs(st.vel - g["vel"]).max() < 1e-4 * np.abs(g["vel"]).max()


@pytest.mark.parametrize("n", [2, 3, 33, 64, 65, 256, 1000])
@pytest.mark.parametrize("tpl", [0, 1, 2])
def test_small_sizes(cuda_dev, orc, n, tpl):
    _, bhmod, ic, _ = _mods()
    pos, _, mass = ic.exponential_disk(n, seed=n)
    pos, mass = _f32(pos), _f32(mass)
    b, a = _run(bhmod, pos, mass, cuda_dev, tpl=tpl)
    ref, tree, _ = orc.bh_compute(pos, mass, 0.5, 0.05, b.G)
    t = b.tree_arrays()
    np.testing.assert_array_equal(t["order"], tree["order"])
    np.testing.assert_array_equal(t["parent"], tree["parent"])
    _check_acc(a, ref)


@pytest.mark.parametrize("n", [2, 2047, 2048, 2049, 4095, 4096, 4097, 32767, 32768, 32769, 40000])
@pytest.mark.parametrize("bits", [21, 10])
def test_sort_sizes_at_tile_edges(cuda_dev, orc, n, bits):
    """Keys, order and topology at the radix sort's tile edges (2,048 keys
    per CTA) against numpy's stable argsort; duplicate positions exercise
    the stable order of equal keys."""
    _, bhmod, ic, _ = _mods()
    pos, _, mass = ic.exponential_disk(n, seed=7)
    pos, mass = _f32(pos), _f32(mass)
    if n > 100:
        pos[n // 2: n // 2 + 50] = pos[0]  # equal keys
    b, _ = _run(bhmod, pos, mass, cuda_dev, bits=bits, tpl=-1)
    t = b.tree_arrays()
    codes = orc.morton_codes(pos, bits)
    order = orc.stable_argsort(codes)
    np.testing.assert_array_equal(t["code"], codes[order])
    np.testing.assert_array_equal(t["order"], order)
    if n >= 2:
        left, right, parent = orc.build_radix(codes[order])
        np.testing.assert_array_equal(t["left"], left)
        np.testing.assert_array_equal(t["parent"], parent)
    assert b.diag()["bad_tree"] == 0
    b.close()


@pytest.mark.parametrize("bits", [21, 10])
def test_sort_many_tiles(cuda_dev, orc, bits):
    """3M keys: 1,465 tiles, more than the CTAs resident at once, so tiles
    look back across CTAs that started in later waves.  Keys and order
    against numpy's stable argsort; no look-back wait runs out."""
    _, bhmod, ic, _ = _mods()
    n = 3_000_000
    pos, _, mass = ic.exponential_disk(n, seed=11)
    pos, mass = _f32(pos), _f32(mass)
    pos[1000:1300] = pos[5]  # a run of equal keys spanning tiles
    b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, key_bits=bits, device=cuda_dev)
    b.build(_xm(pos, mass, cuda_dev))
    codes = orc.morton_codes(pos, bits)
    order = np.argsort(codes, kind="stable")
    np.testing.assert_array_equal(b.export("order"), order)
    np.testing.assert_array_equal(b.export("code"), codes[order])
    d = b.diag()
    assert d["wait_timeouts"] == 0 and d["bad_tree"] == 0
    b.close()


def test_sort_wait_probe_times_out_and_reports(cuda_dev):
    """The sort's look-back waits are bounded: with tile 0 never published,
    every one of the 256 waits gives up after its poll limit, the call
    returns GB_ETIMEOUT and the context stays usable; with tile 0 published
    first, the look-back returns tile 0's counts."""
    import ctypes

    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    lib = lib_mod.load()
    excl = (ctypes.c_uint32 * 256)()
    timeouts = ctypes.c_uint64(7)
    rc = lib.gb_sort_wait_probe(1000, 1, excl, ctypes.byref(timeouts))
    assert rc == lib_mod.GB_OK
    assert list(excl) == list(range(256)) and timeouts.value == 0
    rc = lib.gb_sort_wait_probe(1000, 0, excl, ctypes.byref(timeouts))
    assert rc == lib_mod.GB_ETIMEOUT
    assert timeouts.value == 256
    assert lib.gb_sort_wait_probe(0, 0, excl, ctypes.byref(timeouts)) == lib_mod.GB_EINVAL
    # The context still works.
    x = torch.arange(8, dtype=torch.float32, device=cuda_dev)
    assert float((x * 2).sum()) == 56.0


def _boundary_positions(n, bits, seed):
    """Coordinates within a few ulps of a key-cell boundary of the FP64
    quantisation: the box is pinned by two anchor particles, the scale is the
    one the reference derives from it (core/solvers/barnes_hut.py:37-45), and
    each coordinate sits at lo + (cell + tiny offset) / scale."""
    rng = np.random.default_rng(seed)
    lo32 = float(np.float32(-3.7))
    hi32 = float(np.float32(-3.7 + 41.3))
    qmax = float((1 << bits) - 1)
    scale = qmax / ((hi32 - lo32) * 1.0000001)
    cell = rng.integers(0, 1 << bits, (n, 3)).astype(np.float64)
    off = rng.normal(0.0, 1e-6, (n, 3)) * rng.choice([1e-2, 1.0, 30.0, 3e3], (n, 3))
    pos = _f32(np.clip(lo32 + (cell + off) / scale, lo32, hi32))
    pos[0], pos[1] = lo32, hi32
    return pos


@pytest.mark.parametrize("bits", [10, 21])
def test_keys_at_quantisation_boundaries(cuda_dev, orc, bits):
    """Keys and order bit-exact against the reference's Morton codes for
    coordinates on key-cell boundaries, where an FP32 evaluation of the
    quantisation would put 24% (10 bits) to 49% (21 bits) of the coordinates
    in the wrong cell."""
    _, bhmod, _, _ = _mods()
    n = 200_000
    pos = _boundary_positions(n, bits, 11 + bits)
    mass = np.full(n, 1.0 / n)
    b, _ = _run(bhmod, pos, mass, cuda_dev, bits=bits, tpl=-1)
    t = b.tree_arrays()
    codes = orc.morton_codes(pos, bits)
    order = orc.stable_argsort(codes)
    np.testing.assert_array_equal(t["code"], codes[order])
    np.testing.assert_array_equal(t["order"], order)
    assert b.diag()["bad_tree"] == 0
    b.close()


@pytest.mark.parametrize("bits,tpl", [(10, 2), (21, 1), (10, 0)])
def test_config2_disk_1m(cuda_dev, orc, bits, tpl):
    """N = 1,000,000 exponential disk (M = 5, Rd = 3, z0 = 0.3, galactic G),
    theta = 0.5, eps = 0.05: keys, order, topology bit-exact at full size;
    forces on 4,096 seeded targets against FP64 direct and FP64 BH."""
    _, bhmod, ic, grav = _mods()
    n = 1_000_000
    pos, _, mass = ic.exponential_disk(n, seed=0)
    pos, mass = _f32(pos), _f32(mass)
    b, a = _run(bhmod, pos, mass, cuda_dev, bits=bits, tpl=tpl)
    t = b.tree_arrays()
    codes = orc.morton_codes(pos, bits)
    order = orc.stable_argsort(codes)
    np.testing.assert_array_equal(t["code"], codes[order])
    np.testing.assert_array_equal(t["order"], order)
    left, right, parent = orc.build_radix(codes[order])
    np.testing.assert_array_equal(t["left"], left)
    np.testing.assert_array_equal(t["right"], right)
    np.testing.assert_array_equal(t["parent"], parent)
    targets = np.random.default_rng(0).choice(n, 4096, replace=False)
    com, nmass, nmin, nmax = orc.summaries(order, pos, mass, parent)
    np.testing.assert_array_equal(t["nmin"], nmin)
    np.testing.assert_array_equal(t["nmax"], nmax)
    np.testing.assert_allclose(t["nmass"], nmass, rtol=5e-6)
    np.testing.assert_allclose(t["com"], com, rtol=0, atol=1e-5 * np.abs(pos).max())
    ref_bh, _ = orc.traverse(pos, order, com, nmass, nmin, nmax, left, right, 0.5, 0.0025, b.G,
                             targets=targets)
    _check_acc(a[targets], ref_bh)
    xm = _xm(pos, mass, cuda_dev)
    direct = grav.acc_fp64_targets(xm, targets, b.G, 0.0025)
    err_gpu = _rel(a[targets], direct)
    err_ref = _rel(ref_bh, direct)
    assert abs(err_gpu.mean() - err_ref.mean()) < 1e-4
    assert err_gpu.mean() < 0.02  # the theta = 0.5 monopole budget


def test_deterministic(cuda_dev):
    _, bhmod, ic, _ = _mods()
    pos, _, mass = ic.exponential_disk(50000, seed=5)
    b, a1 = _run(bhmod, pos, mass, cuda_dev)
    xm = _xm(pos, mass, cuda_dev)
    acc = torch.zeros_like(xm)
    b.compute(xm, acc)
    assert np.array_equal(a1, acc[:, :3].double().cpu().numpy())


def test_bh_kdk_matches_oracle(cuda_dev, orc):
    _, bhmod, ic, _ = _mods()
    n = 3000
    pos, vel, mass = ic.exponential_disk(n, seed=7)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, device=cuda_dev)
    xm = _xm(pos, mass, cuda_dev)
    v4 = torch.zeros_like(xm)
    v4[:, :3] = torch.tensor(vel, dtype=torch.float32)
    acc = torch.zeros_like(xm)
    b.compute(xm, acc)
    dt = 1e-4
    b.kdk(xm, v4, acc, dt, 3)
    p, v = pos.copy(), vel.copy()
    a, _, _ = orc.bh_compute(p, mass, 0.5, 0.05, b.G)
    for _ in range(3):
        v = v + a * (0.5 * dt)
        p = p + v * dt
        a, _, _ = orc.bh_compute(p, mass, 0.5, 0.05, b.G)
        v = v + a * (0.5 * dt)
    gp = xm[:, :3].double().cpu().numpy()
    gv = v4[:, :3].double().cpu().numpy()
    assert np.abs(gp - p).max() < 1e-5 * np.abs(p).max()
    assert np.abs(gv - v).max() < 1e-3 * np.abs(v).max()


def test_bad_arguments(cuda_dev):
    pkg, bhmod, _, _ = _mods()
    b = bhmod.BarnesHut(100, device=cuda_dev)
    with pytest.raises(pkg.GravityError, match="before"):
        b.accel(torch.zeros((100, 4), device=cuda_dev))
    with pytest.raises(ValueError):
        b.compute(torch.zeros((200, 4), device=cuda_dev), torch.zeros((200, 4), device=cuda_dev))
    with pytest.raises(pkg.GravityError, match="key_bits"):
        bhmod.BarnesHut(100, key_bits=16, device=cuda_dev)


def test_traversal_modes_bit_identical(cuda_dev):
    """Per-lane (0) and warp-coherent (1, 2) traversals visit each target's
    nodes in the same order, so their accelerations agree bit for bit."""
    ic = importlib.import_module(PKG_NAME + ".ic")
    bhmod = importlib.import_module(PKG_NAME + ".solvers.barnes_hut")
    pos, _, mass = ic.exponential_disk(20000, seed=12)
    out = []
    for tpl in (0, 1, 2):
        b, a = _run(bhmod, pos, mass, cuda_dev, tpl=tpl)
        out.append(a)
        b.close()
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[1], out[2])


def test_graph_replay_matches_direct_launches(cuda_dev):
    """gb_bh_kdk as a replayed CUDA graph and as direct launches: identical
    trajectories, including a recapture after dt changes."""
    ic = importlib.import_module(PKG_NAME + ".ic")
    bhmod = importlib.import_module(PKG_NAME + ".solvers.barnes_hut")
    pos, vel, mass = ic.exponential_disk(5000, seed=8)
    out = []
    for graph in (True, False):
        xm = _xm(pos, mass, cuda_dev)
        v4 = torch.zeros_like(xm)
        v4[:, :3] = torch.tensor(vel, dtype=torch.float32, device=cuda_dev)
        a4 = torch.zeros_like(xm)
        b = bhmod.BarnesHut(5000, theta=0.5, softening=0.05, device=cuda_dev)
        b.set_graph(graph)
        b.compute(xm, a4)
        b.kdk(xm, v4, a4, 1e-4, 3)
        b.kdk(xm, v4, a4, 2e-4, 2)
        b.kdk(xm, v4, a4, 1e-4, 1)
        torch.cuda.synchronize()
        out.append((xm.clone(), v4.clone(), a4.clone()))
        b.close()
    for u, w in zip(*out):
        assert torch.equal(u, w)


def test_engine_bh_gate_at_256(cuda_dev, orc):
    """Engine(gravity_mode="bh") uses the tree only for n >= 256
    (core/engine.py:75): at n = 255 the accelerations are the direct sum's,
    at n = 256 the tree's (the two differ by the monopole error, about 1e-2
    at theta = 0.6, so each is told apart from the other)."""
    pkg, _, ic, _ = _mods()
    for n in (255, 256):
        pos, vel, mass = ic.exponential_disk(n, seed=21)
        pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
        eng = pkg.Engine(softening=0.05, gravity_mode="bh", theta=0.6, device=cuda_dev)
        eng.load_state(pkg.State.from_arrays(pos, vel, mass))
        a = eng.acc.to_numpy()
        direct = orc.direct_acc(pos, mass, eng.G, 0.0025)
        tree, _, _ = orc.bh_compute(pos, mass, 0.6, 0.05, eng.G)
        err_direct, err_tree = np.median(_rel(a, direct)), np.median(_rel(a, tree))
        if n == 255:
            assert eng._bh is None
            assert err_direct < 1e-5 and err_tree > 1e-4, (err_direct, err_tree)
        else:
            assert eng._bh is not None
            assert err_tree < 1e-5 and err_direct > 1e-4, (err_direct, err_tree)


def test_nonfinite_positions_are_counted_and_reported(cuda_dev):
    """NaN and infinite positions: the keying pass counts them (key 0), the
    call finishes, and a checked call reports them as GB_EINVAL."""
    pkg, bhmod, ic, _ = _mods()
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    n = 5000
    pos, _, mass = ic.exponential_disk(n, seed=31)
    pos = _f32(pos)
    bad = [7, 100, 2500, 4999]
    pos[bad[0], 0] = np.nan
    pos[bad[1], 2] = np.inf
    pos[bad[2]] = np.nan
    pos[bad[3], 1] = -np.inf
    b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, device=cuda_dev)
    xm = _xm(pos, mass, cuda_dev)
    acc = torch.zeros_like(xm)
    b.compute(xm, acc)
    torch.cuda.synchronize()
    assert b.diag(reset=True)["nonfinite"] == len(bad)
    with pytest.raises(pkg.GravityError, match="non-finite") as e:
        b.compute(xm, acc, check=True)
    assert e.value.status == lib_mod.GB_EINVAL
    # A finite system on the same handle passes the check afterwards.
    pos2, _, mass2 = ic.exponential_disk(n, seed=32)
    b.compute(_xm(pos2, mass2, cuda_dev), acc, check=True)
    assert torch.isfinite(acc).all()


@pytest.mark.parametrize("tpl", [0, 1])
def test_checked_calls_report_stack_drops(cuda_dev, orc, tpl):
    """With the check on, a call whose traversal dropped pushes under the
    max_stack rule returns GB_ESTACK (the reference drops them silently,
    core/solvers/barnes_hut.py:212); accelerations are still written, equal to
    the unchecked call's.  An Engine with check=True raises from step()."""
    pkg, bhmod, ic, _ = _mods()
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    g = load_golden("bh")
    pos, mass = g["pos"][:400], g["mass"][:400]
    b, a_plain = _run(bhmod, pos, mass, cuda_dev, bits=21, G=float(g["G"]), max_stack=6, tpl=tpl)
    xm = _xm(pos, mass, cuda_dev)
    acc = torch.zeros_like(xm)
    with pytest.raises(pkg.GravityError, match="max_stack") as e:
        b.compute(xm, acc, check=True)
    assert e.value.status == lib_mod.GB_ESTACK
    assert np.array_equal(acc[:, :3].double().cpu().numpy(), a_plain)
    # The default max_stack drops nothing here: the check passes.
    b2 = bhmod.BarnesHut(400, theta=0.5, softening=0.05, G=float(g["G"]), check=True, device=cuda_dev)
    b2.compute(xm, acc)
    eng = pkg.Engine(softening=0.05, gravity_mode="bh", theta=0.5, max_stack=6, G=float(g["G"]),
                     check=True, device=cuda_dev)
    with pytest.raises(pkg.GravityError, match="max_stack"):
        eng.load_state(pkg.State.from_arrays(pos, np.zeros_like(pos), mass))
    with pytest.raises(pkg.GravityError, match="max_stack"):
        eng.step(1e-4)


# ------------------------------------------------------------- group walk
@pytest.mark.parametrize("n", [2, 3, 33, 1000, 50000])
def test_group_walk_matches_oracle(cuda_dev, orc, n):
    """Traversal shape 3 (group walk): accelerations and tree potentials
    against the oracle's FP64 group walk (the same per-group node sets), with
    the tolerances of the per-particle traversal; repeat calls are
    bit-identical."""
    _, bhmod, ic, _ = _mods()
    pos, _, mass = ic.exponential_disk(n, seed=40 + n)
    pos, mass = _f32(pos), _f32(mass)
    b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, key_bits=10, device=cuda_dev)
    b.set_traversal(3)
    xm = _xm(pos, mass, cuda_dev)
    acc = torch.zeros_like(xm)
    phi = torch.zeros(n, device=cuda_dev)
    b.compute(xm, acc, phi=phi)
    acc2 = torch.zeros_like(xm)
    b.compute(xm, acc2)
    torch.cuda.synchronize()
    assert torch.equal(acc, acc2)
    t = orc.bh_tree(pos, mass, bits=10)
    ref_acc, ref_phi = orc.group_walk(pos, t, 0.5, 0.0025, b.G)
    _check_acc(acc[:, :3].double().cpu().numpy(), ref_acc)
    got = phi.double().cpu().numpy()
    rel = np.abs(got - ref_phi) / np.maximum(np.abs(ref_phi), 1e-300)
    assert np.median(rel) < 1e-5 and np.percentile(rel, 99) < 1e-4 and rel.max() < 1e-2, rel.max()
    d = b.diag()
    assert d["stack_overflow"] == 0 and d["bad_tree"] == 0
    b.close()


def test_group_walk_error_budget_1m(cuda_dev, orc):
    """On the 1M disk workload the group walk's force errors against FP64
    direct sums (4,096 seeded targets) are no worse than the exact
    per-particle traversal's in median and 99th percentile: each group
    accepts a refinement of its targets' node sets."""
    _, bhmod, ic, grav = _mods()
    n = 1_000_000
    pos, _, mass = ic.exponential_disk(n, seed=0)
    pos, mass = _f32(pos), _f32(mass)
    xm = _xm(pos, mass, cuda_dev)
    targets = np.random.default_rng(0).choice(n, 4096, replace=False)
    b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, key_bits=10, device=cuda_dev)
    direct = grav.acc_fp64_targets(xm, targets, b.G, 0.0025)
    err = {}
    for tpl in (1, 3):
        b.set_traversal(tpl)
        acc = torch.zeros_like(xm)
        b.compute(xm, acc)
        err[tpl] = _rel(acc[:, :3].double().cpu().numpy()[targets], direct)
    assert np.median(err[3]) <= np.median(err[1]), (np.median(err[3]), np.median(err[1]))
    assert np.percentile(err[3], 99) <= np.percentile(err[1], 99)
    assert b.diag()["stack_overflow"] == 0
    b.close()


def test_group_walk_kdk_matches_oracle(cuda_dev, orc):
    _, bhmod, ic, _ = _mods()
    n = 3000
    pos, vel, mass = ic.exponential_disk(n, seed=17)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, key_bits=10, device=cuda_dev)
    b.set_traversal(3)
    xm = _xm(pos, mass, cuda_dev)
    v4 = torch.zeros_like(xm)
    v4[:, :3] = torch.tensor(vel, dtype=torch.float32)
    acc = torch.zeros_like(xm)
    b.compute(xm, acc)
    dt = 1e-4
    b.kdk(xm, v4, acc, dt, 3)
    p, v = pos.copy(), vel.copy()
    a, _ = orc.group_walk(p, orc.bh_tree(p, mass, bits=10), 0.5, 0.0025, b.G)
    for _ in range(3):
        v = v + a * (0.5 * dt)
        p = p + v * dt
        a, _ = orc.group_walk(p, orc.bh_tree(p, mass, bits=10), 0.5, 0.0025, b.G)
        v = v + a * (0.5 * dt)
    assert np.abs(xm[:, :3].double().cpu().numpy() - p).max() < 1e-5 * np.abs(p).max()
    assert np.abs(v4[:, :3].double().cpu().numpy() - v).max() < 1e-3 * np.abs(v).max()


def test_engine_group_walk_option(cuda_dev, orc):
    """Engine(gravity_mode="bh", bh_traversal=3) primes and steps with the
    group walk: its accelerations equal the oracle's group walk within the
    traversal tolerances, and one step matches a BarnesHut handle in shape 3
    bit for bit."""
    pkg, bhmod, ic, _ = _mods()
    n = 5000
    pos, vel, mass = ic.exponential_disk(n, seed=5)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    eng = pkg.Engine(softening=0.05, gravity_mode="bh", theta=0.5, key_bits=10, bh_traversal=3,
                     device=cuda_dev)
    eng.load_state(pkg.State.from_arrays(pos, vel, mass))
    ref, _ = orc.group_walk(pos, orc.bh_tree(pos, mass, bits=10), 0.5, 0.0025, eng.G)
    _check_acc(eng.acc.to_numpy(), ref)
    b = bhmod.BarnesHut(n, theta=0.5, softening=0.05, key_bits=10, device=cuda_dev)
    b.set_traversal(3)
    xm = eng.xm.clone()
    v4 = eng.v4.clone()
    a4 = eng.a4.clone()
    eng.step(1e-4)
    b.kdk(xm, v4, a4, 1e-4, 1)
    torch.cuda.synchronize()
    assert torch.equal(eng.xm, xm) and torch.equal(eng.v4, v4) and torch.equal(eng.a4, a4)
    b.close()


@pytest.mark.parametrize("case", ["b21", "b10", "dup"])
def test_group_walk_golden_inputs(cuda_dev, orc, case):
    """The group walk on the reference's fixture inputs (1,200 particles at
    21- and 10-bit keys; 500 particles with duplicated positions, whose
    equal keys exercise the index tie-break): accelerations and potentials
    against the oracle's FP64 group walk on the oracle's tree, whose
    topology the fixtures pin."""
    _, bhmod, _, _ = _mods()
    g = load_golden("bh")
    if case == "dup":
        pos, mass, bits, theta = g["dup_pos"], g["dup_mass"], 10, 0.7
    else:
        pos, mass, bits, theta = g["pos"], g["mass"], int(case[1:]), float(g["theta"])
    pos, mass = _f32(pos), _f32(mass)
    n = pos.shape[0]
    soft = float(g["softening"])
    b = bhmod.BarnesHut(n, theta=theta, softening=soft, key_bits=bits, G=float(g["G"]), device=cuda_dev)
    b.set_traversal(3)
    xm = _xm(pos, mass, cuda_dev)
    acc = torch.zeros_like(xm)
    phi = torch.zeros(n, device=cuda_dev)
    b.compute(xm, acc, phi=phi)
    torch.cuda.synchronize()
    t = orc.bh_tree(pos, mass, bits=bits)
    ref_acc, ref_phi = orc.group_walk(pos, t, theta, soft * soft, float(g["G"]))
    _check_acc(acc[:, :3].double().cpu().numpy(), ref_acc)
    got = phi.double().cpu().numpy()
    rel = np.abs(got - ref_phi) / np.maximum(np.abs(ref_phi), 1e-300)
    assert np.median(rel) < 1e-5 and rel.max() < 1e-2, rel.max()
    d = b.diag()
    assert d["stack_overflow"] == 0 and d["bad_tree"] == 0
    b.close()
