"""The solver mirrors called with the reference's argument lists:
compute_acc_direct(pos, mass, acc, n, G, eps2), kinetic_energy(vel, mass, n),
potential_energy(pos, mass, n, G, eps2) (core/solvers/gravity.py:13-57) and
BarnesHut(n, theta, softening).compute(pos, mass, acc)
(core/solvers/barnes_hut.py:242-259), on numpy arrays, the Engine's
reference-style fields and torch tensors, against the reference's own
outputs (tests/golden/direct.npz).

Tolerances as in the direct tests: accelerations per-particle relative RMS
<= 1e-5 of the FP64 values; energies relative 1e-6 (FP32 pair sums, FP64
reduction)."""
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG_NAME, load_golden

pytestmark = pytest.mark.gpu


def _rel_rms(a, ref):
    rel = np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)
    return float(np.sqrt((rel ** 2).mean()))


def test_direct_mirrors_on_numpy_arrays(cuda_dev):
    grav = importlib.import_module(PKG_NAME + ".solvers.gravity")
    g = load_golden("direct")
    pos, vel, mass = g["pos"], g["vel"], g["mass"]
    n, G, eps2 = pos.shape[0], float(g["G"]), float(g["eps2"])
    acc = np.zeros((n, 3))
    grav.compute_acc_direct(pos, mass, acc, n, G, eps2)
    assert _rel_rms(acc, g["acc"]) < 1e-5
    assert grav.kinetic_energy(vel, mass, n) == pytest.approx(float(g["ke"]), rel=1e-6)
    assert grav.potential_energy(pos, mass, n, G, eps2) == pytest.approx(float(g["pe"]), rel=1e-6)


def test_direct_mirror_on_engine_fields(cuda_dev):
    pkg = importlib.import_module(PKG_NAME)
    grav = importlib.import_module(PKG_NAME + ".solvers.gravity")
    st = importlib.import_module(PKG_NAME + ".state")
    g = load_golden("direct")
    n = g["pos"].shape[0]
    eng = pkg.Engine(softening=0.01, G=1.0, device=cuda_dev)
    eng.load_state(st.State.from_arrays(g["pos"], g["vel"], g["mass"]))
    eng.acc.from_numpy(np.zeros((n, 3)))
    grav.compute_acc_direct(eng.pos, eng.mass, eng.acc, n, float(g["G"]), float(g["eps2"]))
    assert _rel_rms(eng.acc.to_numpy(), g["acc"]) < 1e-5


def test_barnes_hut_reference_form_equals_record_form(cuda_dev):
    bhm = importlib.import_module(PKG_NAME + ".solvers.barnes_hut")
    ic = importlib.import_module(PKG_NAME + ".ic")
    pos, _, mass = ic.exponential_disk(4000, seed=3)
    b = bhm.BarnesHut(4000, theta=0.6, softening=0.1, device=cuda_dev)
    acc_np = np.zeros((4000, 3))
    b.compute(pos, mass, acc_np)
    xm = torch.zeros((4000, 4), dtype=torch.float32, device=cuda_dev)
    xm[:, :3] = torch.tensor(pos, dtype=torch.float32, device=cuda_dev)
    xm[:, 3] = torch.tensor(mass, dtype=torch.float32, device=cuda_dev)
    acc = torch.zeros_like(xm)
    b.compute(xm, acc)
    assert np.array_equal(acc_np, acc[:, :3].double().cpu().numpy())
    # Torch tensors in the reference form, accumulating.
    acc_t = torch.ones((4000, 3), dtype=torch.float32, device=cuda_dev)
    b.compute(xm[:, :3], xm[:, 3], acc_t, accumulate=True)
    ref = 1.0 + acc[:, :3]
    assert torch.allclose(acc_t, ref, rtol=1e-6, atol=1e-6 * float(ref.abs().max()))
    b.close()


@pytest.mark.parametrize("n", [1000, 20000])
def test_separate_kdk_halves_equal_fused_step(cuda_dev, n):
    """Engine.step the reference's way (core/engine.py:108-116): kick(dt/2),
    drift(dt), compute_acc_direct, kick(dt/2) through the mirrors, against
    the fused gb_direct_kdk step: bit for bit."""
    pkg = importlib.import_module(PKG_NAME)
    grav = importlib.import_module(PKG_NAME + ".solvers.gravity")
    lf = importlib.import_module(PKG_NAME + ".integrators.leapfrog")
    st = importlib.import_module(PKG_NAME + ".state")
    ic = importlib.import_module(PKG_NAME + ".ic")
    p, v, m = ic.plummer(n, seed=4)
    s0 = st.State.from_arrays(p, v, m)
    fused = pkg.Engine(softening=0.01, G=1.0, device=cuda_dev)
    fused.load_state(s0)
    split = pkg.Engine(softening=0.01, G=1.0, device=cuda_dev)
    split.load_state(s0)
    dt = 1e-3
    for _ in range(3):
        fused.step(dt)
        lf.kick(split.vel, split.acc, n, 0.5 * dt)
        lf.drift(split.pos, split.vel, n, dt)
        grav.compute_acc_direct(split.xm, split.a4, n, 1.0, 1e-4)
        lf.kick(split.vel, split.acc, n, 0.5 * dt)
    torch.cuda.synchronize()
    assert torch.equal(fused.xm, split.xm)
    assert torch.equal(fused.v4, split.v4)
    assert torch.equal(fused.a4, split.a4)
