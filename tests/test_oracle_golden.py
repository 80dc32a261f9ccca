"""The oracle against the golden fixtures produced by the reference's own code
(tests/golden/gen_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import load_golden


def test_direct_acc_matches_reference(orc):
    g = load_golden("direct")
    acc = orc.direct_acc(g["pos"], g["mass"], float(g["G"]), float(g["eps2"]))
    np.testing.assert_allclose(acc, g["acc"], rtol=1e-12, atol=1e-12)


def test_direct_acc_targets(orc):
    g = load_golden("direct")
    t = np.array([0, 5, 17, 383])
    acc = orc.direct_acc(g["pos"], g["mass"], float(g["G"]), float(g["eps2"]), t)
    np.testing.assert_allclose(acc, g["acc"][t], rtol=1e-12, atol=1e-12)


def test_energies_match_reference(orc):
    g = load_golden("direct")
    ke = orc.kinetic_energy(g["vel"], g["mass"])
    pe = orc.potential_energy(g["pos"], g["mass"], float(g["G"]), float(g["eps2"]))
    assert ke == pytest.approx(float(g["ke"]), rel=1e-13)
    assert pe == pytest.approx(float(g["pe"]), rel=1e-13)
    phi = orc.phi_targets(g["pos"], g["mass"], float(g["eps2"]), np.arange(384))
    pe2 = -0.5 * float(g["G"]) * np.sum(g["mass"] * phi)
    assert pe2 == pytest.approx(float(g["pe"]), rel=1e-13)


def test_engine_kdk_matches_reference(orc):
    g = load_golden("engine_direct")
    G, eps2 = float(g["G"]), float(g["softening"]) ** 2
    acc0 = orc.direct_acc(g["pos0"], g["mass"], G, eps2)
    np.testing.assert_allclose(acc0, g["acc0"], rtol=1e-11, atol=1e-9)
    pos, vel, acc = orc.kdk_direct(g["pos0"], g["vel0"], acc0, g["mass"], G,
                                   eps2, float(g["dt"]), int(g["nsteps"]))
    np.testing.assert_allclose(pos, g["pos"], rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(vel, g["vel"], rtol=1e-10, atol=1e-8)
    np.testing.assert_allclose(acc, g["acc"], rtol=1e-9, atol=1e-6)
    ke = orc.kinetic_energy(vel, g["mass"])
    pe = orc.potential_energy(pos, g["mass"], G, eps2)
    assert ke == pytest.approx(g["e1"][0], rel=1e-11)
    assert pe == pytest.approx(g["e1"][1], rel=1e-11)


@pytest.mark.parametrize("case", ["disk", "plummer", "dups", "same", "plane", "wide"])
@pytest.mark.parametrize("bits", [21, 10])
def test_morton_bit_exact(orc, case, bits):
    g = load_golden("morton")
    pos = g[f"{case}_pos"]
    ref = g[f"{case}_code{bits}"]
    np.testing.assert_array_equal(orc.morton_codes(pos, bits), ref)
    np.testing.assert_array_equal(orc.morton_codes_numpy(pos, bits), ref)
    np.testing.assert_array_equal(orc.stable_argsort(ref), g[f"{case}_order{bits}"])


@pytest.mark.parametrize("bits", [21, 10])
def test_karras_topology_bit_exact(orc, bits):
    g = load_golden("bh")
    pre = f"b{bits}_"
    order = orc.stable_argsort(g[pre + "code"])
    np.testing.assert_array_equal(order, g[pre + "order"])
    left, right, parent = orc.build_radix(g[pre + "code"][order])
    np.testing.assert_array_equal(left, g[pre + "left"])
    np.testing.assert_array_equal(right, g[pre + "right"])
    np.testing.assert_array_equal(parent, g[pre + "parent"])


def test_karras_duplicates_bit_exact(orc):
    g = load_golden("bh")
    codes = orc.morton_codes(g["dup_pos"], 10)
    np.testing.assert_array_equal(codes, g["dup_code"])
    order = orc.stable_argsort(codes)
    left, right, parent = orc.build_radix(codes[order])
    np.testing.assert_array_equal(left, g["dup_left"])
    np.testing.assert_array_equal(right, g["dup_right"])
    np.testing.assert_array_equal(parent, g["dup_parent"])


@pytest.mark.parametrize("bits", [21, 10])
def test_summaries_and_traversal(orc, bits):
    g = load_golden("bh")
    pre = f"b{bits}_"
    t = orc.bh_tree(g["pos"], g["mass"], bits)
    np.testing.assert_array_equal(t["nmin"], g[pre + "nmin"])
    np.testing.assert_array_equal(t["nmax"], g[pre + "nmax"])
    np.testing.assert_allclose(t["nmass"], g[pre + "nmass"], rtol=1e-14)
    np.testing.assert_allclose(t["com"], g[pre + "com"], rtol=1e-12, atol=1e-12)
    acc, dropped = orc.traverse(g["pos"], t["order"], t["com"], t["nmass"],
                                t["nmin"], t["nmax"], t["left"], t["right"],
                                float(g["theta"]), float(g["softening"]) ** 2,
                                float(g["G"]))
    assert dropped == 0
    np.testing.assert_allclose(acc, g[pre + "acc"], rtol=1e-9, atol=1e-7)


def test_bh_compute_and_stack_drop(orc):
    g = load_golden("bh")
    acc, _, dropped = orc.bh_compute(g["pos"], g["mass"], 0.5, 0.05, float(g["G"]))
    np.testing.assert_allclose(acc, g["compute_acc"], rtol=1e-9, atol=1e-7)
    acc6, _, dropped6 = orc.bh_compute(g["pos"][:400], g["mass"][:400], 0.5,
                                       0.05, float(g["G"]), max_stack=6)
    assert dropped6 > 0
    np.testing.assert_allclose(acc6, g["stk6_acc"], rtol=1e-9, atol=1e-7)


def test_dup_traversal(orc):
    g = load_golden("bh")
    acc, _, _ = orc.bh_compute(g["dup_pos"], g["dup_mass"], 0.7, 0.05,
                               float(g["G"]), bits=10)
    np.testing.assert_allclose(acc, g["dup_acc"], rtol=1e-9, atol=1e-7)


def test_engine_bh_matches_reference(orc):
    g = load_golden("engine_bh")
    G, eps = float(g["G"]), float(g["softening"])
    acc0, _, _ = orc.bh_compute(g["pos0"], g["mass"], float(g["theta"]), eps, G)
    np.testing.assert_allclose(acc0, g["acc0"], rtol=1e-9, atol=1e-6)
    pos, vel, acc = g["pos0"].copy(), g["vel0"].copy(), acc0
    dt = float(g["dt"])
    for _ in range(int(g["nsteps"])):
        vel = vel + acc * (0.5 * dt)
        pos = pos + vel * dt
        acc, _, _ = orc.bh_compute(pos, g["mass"], float(g["theta"]), eps, G)
        vel = vel + acc * (0.5 * dt)
    np.testing.assert_allclose(pos, g["pos"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(vel, g["vel"], rtol=1e-9, atol=1e-7)


def _potential(g, name):
    return {k: g[f"{name}_{k}"].item() for k in ("M_d", "a", "b", "M_h", "a_h", "is_hernquist", "smbh_mass")}


@pytest.mark.parametrize("name", ["mn_plummer", "hernquist_smbh", "mn_hernquist_smbh"])
def test_analytic_potential_matches_reference(orc, name):
    """grav_analytic / add_analytic bit for bit; add_grav_ext to FP64
    rounding of its self-gravity sum."""
    g = load_golden("analytic")
    pot = _potential(g, name)
    G, eps2 = float(g["G"]), float(g["eps2"])
    acc = orc.analytic_acc(g["pos"], G, pot, g["acc0"])
    np.testing.assert_array_equal(acc, g[f"{name}_grav_analytic"])
    np.testing.assert_array_equal(acc, g[f"{name}_add_analytic"])
    ext = orc.grav_ext_acc(g["pos"], g["mass"], G, eps2, pot, g["acc0"])
    np.testing.assert_allclose(ext, g[f"{name}_add_grav_ext"], rtol=1e-13, atol=1e-10)


def test_neighbor_grid_matches_reference(orc):
    """NeighborGrid.rebuild / rebuild_all: every output bit for bit on the
    seven fixture cases (the no-gas case runs on the disk case's grid)."""
    g = load_golden("neighbor_grid")
    prev = None
    for name in g["names"]:
        star = g.get(f"{name}_is_star")
        r = orc.grid_rebuild(g[f"{name}_pos"], g[f"{name}_h"], star, float(g[f"{name}_min_radius"]),
                             state=prev if name == "nogas" else None)
        assert r["ngas"] == int(g[f"{name}_ngas"]), name
        np.testing.assert_array_equal(r["gsort"], g[f"{name}_gsort"])
        np.testing.assert_array_equal(r["cell_start"], g[f"{name}_cell_start"])
        np.testing.assert_array_equal(r["dims"], g[f"{name}_dims"])
        np.testing.assert_array_equal(r["lo"], g[f"{name}_lo"])
        assert r["inv_cell"] == float(g[f"{name}_inv_cell"])
        if name == "disk":
            prev = r
