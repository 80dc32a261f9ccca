"""Generate the golden fixtures in this directory by running the REFERENCE's own
hot-path Python code (Khaserdene/real-astronomy-simulation) on the host.

Taichi is not installable offline, so the reference modules are imported under
``_taichi_stub`` (kernels run as serial Python over numpy fields).  The only
source change is ``rewrite_atomics`` applied to ``_accumulate``
(core/solvers/barnes_hut.py:143-166), turning ``ti.atomic_add/min/max`` on a
field element into the equivalent in-place update.

Run from the repository root, in a container where the reference is mounted,
with the reference's root directory as the first argument:

    python tests/golden/gen_golden.py <reference root> [generator names...]

Inputs are rounded to float32 first (the GPU engine stores float32), then
passed to the reference as float64, so the fixtures describe the reference's
arithmetic on exactly the values the device sees.  Outputs are written as
compressed ``.npz`` files next to this script; the tests read only those.
"""
from __future__ import annotations

import inspect
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _load_reference(ref_root: str):
    sys.dont_write_bytecode = True
    sys.path.insert(0, HERE)
    import _taichi_stub
    _taichi_stub.install()
    sys.path.insert(0, ref_root)
    import core.units as units
    import core.solvers.gravity as gravity
    import core.solvers.barnes_hut as bh
    import core.integrators.leapfrog as leapfrog
    import core.ic.plummer as plummer
    import core.ic.disk as disk
    import core.engine as engine
    import core.living_galaxy_engine as living
    import core.gas_disk_engine as gasdisk
    import core.solvers.neighbor_grid as ngrid
    # _accumulate: atomics -> in-place updates (the only source rewrite).
    src = _taichi_stub.rewrite_atomics(inspect.getsource(bh._accumulate))
    exec(compile(src, bh.__file__, "exec"), bh.__dict__)
    return dict(units=units, gravity=gravity, bh=bh, leapfrog=leapfrog,
                plummer=plummer, disk=disk, engine=engine, living=living,
                gasdisk=gasdisk, ngrid=ngrid, stub=_taichi_stub)


def _f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def _field_from(stub, arr, dtype="f64"):
    arr = np.asarray(arr)
    f = stub._field(dtype, arr.shape)
    f.from_numpy(arr)
    return f


def gen_plummer_ic(R, out):
    """make_plummer with G patched to 1 (core/ic/plummer.py:19-66)."""
    pl = R["plummer"]
    old = pl.G
    pl.G = 1.0
    try:
        s0 = pl.make_plummer(n=1000, total_mass=1.0, scale_radius=1.0, seed=0)
        s1 = pl.make_plummer(n=257, total_mass=2.5, scale_radius=0.7, seed=11)
    finally:
        pl.G = old
    out["plummer_ic"] = dict(pos0=s0.pos, vel0=s0.vel, mass0=s0.mass,
                             pos1=s1.pos, vel1=s1.vel, mass1=s1.mass)


def gen_direct(R, out):
    """compute_acc_direct / kinetic_energy / potential_energy
    (core/solvers/gravity.py:13-57) on a float32-rounded Plummer sphere."""
    pl, grav, stub = R["plummer"], R["gravity"], R["stub"]
    old = pl.G
    pl.G = 1.0
    try:
        s = pl.make_plummer(n=384, total_mass=1.0, scale_radius=1.0, seed=5)
    finally:
        pl.G = old
    pos, vel, mass = _f32(s.pos), _f32(s.vel), _f32(s.mass)
    n = pos.shape[0]
    G, eps2 = 1.0, 0.01 ** 2
    fp = _field_from(stub, pos)
    fm = _field_from(stub, mass)
    fv = _field_from(stub, vel)
    fa = stub._field("f64", (n, 3))
    grav.compute_acc_direct(fp, fm, fa, n, G, eps2)
    ke = grav.kinetic_energy(fv, fm, n)
    pe = grav.potential_energy(fp, fm, n, G, eps2)
    out["direct"] = dict(pos=pos, vel=vel, mass=mass, G=G, eps2=eps2,
                         acc=fa.to_numpy(), ke=ke, pe=pe)


def gen_engine_direct(R, out):
    """Engine(softening=0.05) KDK stepping (core/engine.py:108-116) with the
    reference's own G = 43009.1725 (core/units.py:21)."""
    pl, eng_mod, units = R["plummer"], R["engine"], R["units"]
    s = pl.make_plummer(n=48, total_mass=10.0, scale_radius=1.0, seed=42)
    s.pos, s.vel, s.mass = _f32(s.pos), _f32(s.vel), _f32(s.mass)
    eng = eng_mod.Engine(softening=0.05)
    eng.load_state(s)
    acc0 = eng.acc.to_numpy()
    e0 = eng.energies()
    dt, nsteps = 3e-5, 25
    for _ in range(nsteps):
        eng.step(dt)
    st = eng.to_state()
    out["engine_direct"] = dict(
        pos0=s.pos, vel0=s.vel, mass=s.mass, acc0=acc0, dt=dt,
        nsteps=nsteps, softening=0.05, G=units.G, pos=st.pos, vel=st.vel,
        acc=eng.acc.to_numpy(), e0=np.array(e0), e1=np.array(eng.energies()),
        time=eng.time, step=eng.step_count)


def _disk_positions(R, n, seed):
    dk = R["disk"]
    g = dk.make_disk_galaxy(n_disk=n // 2, n_halo=n - n // 2, seed=seed)
    return _f32(g.pos), _f32(g.mass)


def gen_morton(R, out):
    """morton_codes (core/solvers/barnes_hut.py:27-46) at bits=21 and bits=10,
    plus the stable argsort of core/solvers/barnes_hut.py:247."""
    bh = R["bh"]
    rng = np.random.default_rng(123)
    cases = {}
    p, _ = _disk_positions(R, 8192, seed=3)
    cases["disk"] = p
    pl = R["plummer"]
    cases["plummer"] = _f32(pl.make_plummer(n=8192, seed=4).pos)
    # Heavy duplicates: 600 distinct points each repeated, shuffled.
    base = _f32(rng.normal(size=(600, 3)))
    cases["dups"] = base[rng.integers(0, 600, size=4096)]
    # Degenerate: all points equal (span == 0 -> 1.0 branch, :42).
    cases["same"] = np.tile(_f32([[1.5, -2.25, 0.125]]), (64, 1))
    # Planar + tiny extents + negative coordinates.
    q = _f32(rng.uniform(-1e-3, 1e-3, size=(2048, 3)))
    q[:, 2] = -7.0
    cases["plane"] = q
    # Wide dynamic range.
    cases["wide"] = _f32(rng.standard_cauchy(size=(4096, 3)) * 50.0)
    res = {}
    for name, pos in cases.items():
        res[f"{name}_pos"] = pos
        for bits in (21, 10):
            c = bh.morton_codes(pos, bits=bits)
            res[f"{name}_code{bits}"] = c
            res[f"{name}_order{bits}"] = np.argsort(c, kind="stable").astype(np.int32)
    out["morton"] = res


def _bh_pipeline(R, pos, mass, theta, softening, bits, max_stack=64):
    """The body of BarnesHut.compute (core/solvers/barnes_hut.py:242-259) with
    the key width as a parameter (the reference hard-codes bits=21 at :246)."""
    bh, stub = R["bh"], R["stub"]
    n = pos.shape[0]
    B = bh.BarnesHut(n, theta=theta, softening=softening, max_stack=max_stack)
    fp = _field_from(stub, pos)
    fm = _field_from(stub, mass)
    fa = stub._field("f64", (n, 3))
    codes = bh.morton_codes(pos, bits=bits)
    order = np.argsort(codes, kind="stable").astype(np.int32)
    B.code.from_numpy(codes[order].astype(np.int64))
    B.order.from_numpy(order)
    B.parent.from_numpy(np.full(2 * n - 1, -1, np.int32))
    bh._build_radix(B.code, B.left, B.right, B.parent, n)
    bh._leaf_init(B.order, fp, fm, B.com, B.nmass, B.nmom, B.nmin, B.nmax, n)
    bh._accumulate(B.parent, B.com, B.nmass, B.nmom, B.nmin, B.nmax, n)
    bh._finalize(B.com, B.nmass, B.nmom, n)
    bh._traverse(fp, B.order, B.com, B.nmass, B.nmin, B.nmax, B.left, B.right,
                 fa, B.stack, n, n, B.theta2, B.eps2, B.max_stack)
    return dict(code=codes, order=order, left=B.left.to_numpy(),
                right=B.right.to_numpy(), parent=B.parent.to_numpy(),
                com=B.com.to_numpy(), nmass=B.nmass.to_numpy(),
                nmin=B.nmin.to_numpy(), nmax=B.nmax.to_numpy(),
                acc=fa.to_numpy())


def gen_bh(R, out):
    """LBVH Barnes-Hut stages on a disk sample (G = 43009.1725 is compiled
    into _traverse, core/solvers/barnes_hut.py:202,210)."""
    bh, stub = R["bh"], R["stub"]
    pos, mass = _disk_positions(R, 1200, seed=9)
    res = {"pos": pos, "mass": mass, "theta": 0.5, "softening": 0.05,
           "G": R["units"].G}
    for bits in (21, 10):
        r = _bh_pipeline(R, pos, mass, 0.5, 0.05, bits)
        for k, v in r.items():
            res[f"b{bits}_{k}"] = v
    # BarnesHut.compute itself (bits=21 path), to pin the pipeline above.
    n = pos.shape[0]
    B = bh.BarnesHut(n, theta=0.5, softening=0.05)
    fa = stub._field("f64", (n, 3))
    B.compute(_field_from(stub, pos), _field_from(stub, mass), fa)
    res["compute_acc"] = fa.to_numpy()
    # A tiny stack exercises the silent drop at :212.
    r = _bh_pipeline(R, pos[:400], mass[:400], 0.5, 0.05, 21, max_stack=6)
    res["stk6_acc"] = r["acc"]
    # Duplicate-heavy input: equal codes use the index tie-break (:77-78).
    rng = np.random.default_rng(77)
    base = _f32(rng.normal(size=(90, 3)))
    dpos = base[rng.integers(0, 90, size=500)]
    dmass = _f32(rng.uniform(0.5, 1.5, size=500) * 1e-3)
    r = _bh_pipeline(R, dpos, dmass, 0.7, 0.05, 10)
    res["dup_pos"], res["dup_mass"] = dpos, dmass
    for k, v in r.items():
        res[f"dup_{k}"] = v
    out["bh"] = res


def gen_engine_bh(R, out):
    """Engine(gravity_mode="bh") stepping (core/engine.py:74-80,101-116)."""
    eng_mod, units = R["engine"], R["units"]
    dk = R["disk"]
    g = dk.make_disk_galaxy(n_disk=160, n_halo=140, seed=21)
    g.pos, g.vel, g.mass = _f32(g.pos), _f32(g.vel), _f32(g.mass)
    eng = eng_mod.Engine(softening=0.1, gravity_mode="bh", theta=0.6)
    eng.load_state(g)
    acc0 = eng.acc.to_numpy()
    dt, nsteps = 1e-4, 4
    for _ in range(nsteps):
        eng.step(dt)
    out["engine_bh"] = dict(pos0=g.pos, vel0=g.vel, mass=g.mass, acc0=acc0,
                            dt=dt, nsteps=nsteps, softening=0.1, theta=0.6,
                            G=units.G, pos=eng.pos.to_numpy(),
                            vel=eng.vel.to_numpy(), acc=eng.acc.to_numpy())


# Potentials of the fixtures: the engines' default (core/gas_disk_engine.py:
# 130), the giant-impact scenario's halo + black hole (core/scenarios.py:331)
# and both together.
POTENTIALS = {
    "mn_plummer": dict(M_d=5.0, a=3.0, b=0.3, M_h=12.0, a_h=8.0,
                       is_hernquist=0, smbh_mass=0.0),
    "hernquist_smbh": dict(M_d=0.0, a=1.0, b=1.0, M_h=40.0, a_h=15.0,
                           is_hernquist=1, smbh_mass=0.1),
    "mn_hernquist_smbh": dict(M_d=5.0, a=3.0, b=0.3, M_h=40.0, a_h=15.0,
                              is_hernquist=1, smbh_mass=0.1),
}


def gen_analytic(R, out):
    """The analytic galaxy potential added after self-gravity:
    grav_analytic (core/living_galaxy_engine.py:124-151), add_analytic
    (core/gas_disk_engine.py:54-81) and add_grav_ext (self-gravity +
    analytic, :20-51), each adding into an acc array that already holds
    values.  Particle 0 sits at the origin and particle 1 on the z axis."""
    lg, gd, stub, units = R["living"], R["gasdisk"], R["stub"], R["units"]
    pos, mass = _disk_positions(R, 240, seed=31)
    pos[0] = 0.0
    pos[1, :2] = 0.0
    n = pos.shape[0]
    rng = np.random.default_rng(32)
    acc0 = _f32(rng.normal(0.0, 1.0e4, (n, 3)))
    eps2 = 0.05 ** 2
    d = dict(pos=pos, mass=mass, acc0=acc0, G=units.G, eps2=eps2)
    fp, fm = _field_from(stub, pos), _field_from(stub, mass)
    for name, pot in POTENTIALS.items():
        args = (pot["M_d"], pot["a"], pot["b"], pot["M_h"], pot["a_h"],
                pot["is_hernquist"], pot["smbh_mass"])
        for k, v in pot.items():
            d[f"{name}_{k}"] = v
        fa = _field_from(stub, acc0)
        lg.grav_analytic(fp, fa, n, *args)
        d[f"{name}_grav_analytic"] = fa.to_numpy()
        fa = _field_from(stub, acc0)
        gd.add_analytic(fp, fa, n, *args)
        d[f"{name}_add_analytic"] = fa.to_numpy()
        fa = _field_from(stub, acc0)
        gd.add_grav_ext(fp, fm, fa, n, eps2, *args)
        d[f"{name}_add_grav_ext"] = fa.to_numpy()
    d["names"] = np.array(list(POTENTIALS))
    out["analytic"] = d


def gen_neighbor_grid(R, out):
    """NeighborGrid.rebuild / rebuild_all (core/solvers/neighbor_grid.py:
    35-136) on float32-rounded inputs.  Cases: a disk with 30% stars; the
    same with rebuild_all and a dominant min_radius; smoothing lengths so
    small that the cell-growth loop runs; a rebuild without gas after a
    normal one (the fields must stay as they were); points on exact cell
    boundaries with duplicates; zero smoothing lengths (cell falls back to
    1); a single gas particle."""
    ng, stub = R["ngrid"], R["stub"]
    rng = np.random.default_rng(41)
    d = {}

    def run(name, pos, h, is_star=None, min_radius=0.0, grid=None):
        n = pos.shape[0]
        g = grid if grid is not None else ng.NeighborGrid(n, min_radius=min_radius)
        fp, fh = _field_from(stub, pos), _field_from(stub, h)
        if is_star is None:
            ngas = g.rebuild_all(fp, fh)
        else:
            ngas = g.rebuild(fp, fh, _field_from(stub, is_star, "i32"))
        d[f"{name}_pos"], d[f"{name}_h"] = pos, h
        if is_star is not None:
            d[f"{name}_is_star"] = is_star
        d[f"{name}_min_radius"] = min_radius
        d[f"{name}_ngas"] = ngas
        d[f"{name}_gsort"] = g.gsort.to_numpy()
        d[f"{name}_cell_start"] = g.cell_start.to_numpy()
        d[f"{name}_dims"] = np.array([g.nx, g.ny, g.nz], np.int64)
        d[f"{name}_lo"] = np.array(g.lo, np.float64)
        d[f"{name}_inv_cell"] = g.inv_cell
        return g

    pos, _ = _disk_positions(R, 3000, seed=43)
    h = _f32(rng.lognormal(np.log(0.3), 0.4, 3000))
    star = (rng.random(3000) < 0.3).astype(np.int32)
    g = run("disk", pos, h, star)
    run("disk_all", pos, h, None, min_radius=1.5)
    run("tiny_h", _f32(rng.normal(0.0, 2.0, (500, 3))), _f32(np.full(500, 1e-4)), None)
    nostar = np.ones(3000, np.int32)
    run("nogas", pos, h, nostar, grid=g)  # after "disk": fields unchanged
    lat = _f32(np.stack(np.meshgrid(np.arange(8), np.arange(5), np.arange(3), indexing="ij"),
                        -1).reshape(-1, 3) * 0.5)
    lat = np.concatenate([lat, lat[::7]])  # duplicates
    run("lattice", lat, _f32(np.full(lat.shape[0], 0.25)), np.zeros(lat.shape[0], np.int32))
    run("zero_h", pos[:400], _f32(np.zeros(400)), star[:400])
    one = np.ones(50, np.int32)
    one[17] = 0
    run("single_gas", pos[:50], h[:50], one)
    d["names"] = np.array(["disk", "disk_all", "tiny_h", "nogas", "lattice", "zero_h", "single_gas"])
    out["neighbor_grid"] = d


GENERATORS = (gen_plummer_ic, gen_direct, gen_engine_direct, gen_morton,
              gen_bh, gen_engine_bh, gen_analytic, gen_neighbor_grid)


def main(argv):
    """argv: [script, reference root, generator names...]; no names runs
    every generator."""
    if len(argv) < 2:
        sys.exit("usage: gen_golden.py <reference root> [generator names...]")
    ref_root = argv[1]
    R = _load_reference(ref_root)
    out = {}
    wanted = set(argv[2:])
    for fn in GENERATORS:
        if wanted and fn.__name__ not in wanted:
            continue
        t0 = time.time()
        fn(R, out)
        print(f"{fn.__name__}: {time.time() - t0:.1f}s", flush=True)
    for name, d in out.items():
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in d.items()})
        print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KB)")


if __name__ == "__main__":
    main(sys.argv)
