"""Hand-written adjoint of the direct-sum KDK leapfrog against a dense FP64
torch-autograd reference and FP64 central finite differences (the C oracle's
KDK), on an N = 256 exponential disk (Rd = 3 kpc, eps = 0.05 kpc, galactic
G, dt = 1e-3, 200 steps, checkpoint every 20) whose particles have the mass
of the N = 65,536 workload's (total mass 5 * 256 / 65536).  With the full
5e10 Msun on 256 particles, close encounters at eps = 0.05 make the step map
so sensitive that central differences do not converge at any step size, so
that system cannot check a gradient.

Tolerances: the device gradients come from FP32 forces and FP32 adjoint
sums, so their relative L2 distance from the FP64 gradients is set to 2e-3,
directional derivatives to 3e-3; checkpoint intervals must not change the
gradients at all (the backward pass replays the forward steps bit for bit).
"""
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG_NAME

pytestmark = pytest.mark.gpu

G = 43009.1725
EPS = 0.05
DT = 1e-3


def _mods():
    return (importlib.import_module(PKG_NAME + ".adjoint"), importlib.import_module(PKG_NAME + ".ic"),
            importlib.import_module(PKG_NAME + ".solvers.gravity"))


def _problem(n=256, seed=3):
    _, ic, _ = _mods()
    p, v, m = ic.exponential_disk(n, total_mass=5.0 * n / 65536, seed=seed)
    f = lambda a: a.astype(np.float32).astype(np.float64)
    p, v, m = f(p), f(v), f(m)
    rng = np.random.default_rng(seed + 1)
    target = p + rng.normal(0.0, 0.05, size=p.shape)
    return p, v, m, target


def dense_kdk(x, v, m, nsteps, eps2=EPS * EPS):
    """FP64 torch reference of nsteps KDK steps with dense pairwise forces."""
    def acc(x):
        d = x[None, :, :] - x[:, None, :]  # d[i, j] = x_j - x_i
        r2 = (d * d).sum(-1) + eps2
        return G * (m[None, :, None] * d * (r2 ** -1.5)[..., None]).sum(1)

    a = acc(x)
    for _ in range(nsteps):
        vh = v + 0.5 * DT * a
        x = x + DT * vh
        a = acc(x)
        v = vh + 0.5 * DT * a
    return x, v


def _loss(x, v, target):
    return ((x - target) ** 2).mean() + 1e-6 * (v ** 2).mean()


# Adjoint pair evaluations: (symmetric, packed) arguments of adjoint.simulate.
FORMS = {"packed": (True, True), "scalar": (True, False), "per_target": (False, True)}


def _device_grads(p, v, m, target, nsteps, every, dev, form="packed"):
    adj, _, grav = _mods()
    symmetric, packed = FORMS[form]
    x0 = torch.tensor(p, dtype=torch.float32, device=dev, requires_grad=True)
    v0 = torch.tensor(v, dtype=torch.float32, device=dev, requires_grad=True)
    m0 = torch.tensor(m, dtype=torch.float32, device=dev, requires_grad=True)
    solver = grav.DirectGravity(p.shape[0], dev)
    xT, vT = adj.simulate(x0, v0, m0, G=G, softening=EPS, dt=DT, nsteps=nsteps,
                          checkpoint_every=every, solver=solver, symmetric=symmetric, packed=packed)
    loss = _loss(xT.double(), vT.double(), torch.tensor(target, device=dev))
    loss.backward()
    return [t.grad.double().cpu().numpy() for t in (x0, v0, m0)], float(loss.detach())


def _dense_grads(p, v, m, target, nsteps):
    x0 = torch.tensor(p, requires_grad=True)
    v0 = torch.tensor(v, requires_grad=True)
    m0 = torch.tensor(m, requires_grad=True)
    xT, vT = dense_kdk(x0, v0, m0, nsteps)
    loss = _loss(xT, vT, torch.tensor(target))
    loss.backward()
    return [t.grad.numpy() for t in (x0, v0, m0)], float(loss.detach())


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("form", list(FORMS))
def test_adjoint_matches_dense_autograd(cuda_dev, form):
    p, v, m, target = _problem()
    g_dev, l_dev = _device_grads(p, v, m, target, 200, 20, cuda_dev, form)
    g_ref, l_ref = _dense_grads(p, v, m, target, 200)
    assert abs(l_dev - l_ref) < 1e-4 * abs(l_ref)
    for name, a, b in zip(("x0", "v0", "m"), g_dev, g_ref):
        assert _rel(a, b) < 2e-3, (name, _rel(a, b))


@pytest.mark.parametrize("form", list(FORMS))
def test_adjoint_ragged_tiles_match_dense(cuda_dev, form):
    """N = 520: diagonal, off-diagonal and padded tile pairs of the symmetric
    forms (two full 256-particle tiles and a partial one; one full
    512-particle tile and a partial one)."""
    p, v, m, target = _problem(n=520, seed=13)
    g_dev, _ = _device_grads(p, v, m, target, 30, 10, cuda_dev, form)
    g_ref, _ = _dense_grads(p, v, m, target, 30)
    for name, a, b in zip(("x0", "v0", "m"), g_dev, g_ref):
        assert _rel(a, b) < 2e-3, (name, _rel(a, b))


@pytest.mark.parametrize("form", list(FORMS))
def test_checkpoint_interval_does_not_change_gradients(cuda_dev, form):
    p, v, m, target = _problem(n=300, seed=5)
    base, _ = _device_grads(p, v, m, target, 24, 24, cuda_dev, form)
    for every in (1, 5, 7):
        g, _ = _device_grads(p, v, m, target, 24, every, cuda_dev, form)
        for a, b in zip(g, base):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("form", ["packed", "scalar"])
def test_symmetric_matches_per_target_form(cuda_dev, form):
    p, v, m, target = _problem(n=3000, seed=17)
    g1, _ = _device_grads(p, v, m, target, 10, 5, cuda_dev, form)
    g0, _ = _device_grads(p, v, m, target, 10, 5, cuda_dev, "per_target")
    for a, b in zip(g1, g0):
        assert _rel(a, b) < 1e-4


@pytest.mark.parametrize("n", [65536, 80000])
def test_adjoint_step_forms_agree_at_large_n(cuda_dev, n):
    """One backward step of each pair evaluation on the same inputs.  The
    packed form splits tile pairs into 2 source slices at N = 65,536 and
    none at N = 80,000 (the small cases above use 4 slices)."""
    _, ic, grav = _mods()
    lib = importlib.import_module(PKG_NAME + "._lib")
    p, _, m = ic.exponential_disk(n, total_mass=5.0, seed=2)
    xm = torch.zeros((n, 4), dtype=torch.float32, device=cuda_dev)
    xm[:, :3] = torch.tensor(p, device=cuda_dev)
    xm[:, 3] = torch.tensor(m, device=cuda_dev)
    gen = torch.Generator().manual_seed(4)
    base = [torch.randn((n, 4), generator=gen).to(cuda_dev) for _ in range(3)]
    solver = grav.DirectGravity(n, cuda_dev)
    stream = torch.cuda.current_stream(cuda_dev).cuda_stream
    out = {}
    for variant in (2, 1, 0):
        lib.call("gb_adjoint_set_variant", solver.handle, variant)
        lx, lv, la = [b.clone() for b in base]
        lm = torch.zeros(n, dtype=torch.float32, device=cuda_dev)
        lib.call("gb_adjoint_step", solver.handle, xm.data_ptr(), lx.data_ptr(), lv.data_ptr(), la.data_ptr(),
                 lm.data_ptr(), n, G, EPS * EPS, DT, 0, stream)
        out[variant] = [t.double().cpu().numpy() for t in (lx[:, :3], lv[:, :3], la[:, :3], lm)]
    solver.close()
    for variant in (2, 1):
        for a, b in zip(out[variant], out[0]):
            assert np.all(np.isfinite(a))
            assert _rel(a, b) < 1e-5, (variant, _rel(a, b))


def test_adjoint_matches_fp64_finite_differences(cuda_dev, orc):
    """Directional derivatives of the FP64 oracle's KDK (central differences)
    against the device gradient projected on random directions."""
    p, v, m, target = _problem(n=256, seed=7)
    nsteps = 200
    g_dev, _ = _device_grads(p, v, m, target, nsteps, 20, cuda_dev)

    def loss(pp, vv, mm):
        a0 = orc.direct_acc(pp, mm, G, EPS * EPS)
        x, vT, _ = orc.kdk_direct(pp, vv, a0, mm, G, EPS * EPS, DT, nsteps)
        return ((x - target) ** 2).mean() + 1e-6 * (vT ** 2).mean()

    rng = np.random.default_rng(11)
    for which, base in enumerate((p, v, m)):
        for _ in range(2):
            d = rng.normal(size=base.shape)
            h = 1e-6 * np.abs(base).max()
            args_p = [p, v, m]
            args_m = [p, v, m]
            args_p[which] = base + h * d
            args_m[which] = base - h * d
            fd = (loss(*args_p) - loss(*args_m)) / (2 * h)
            an = float((g_dev[which] * d).sum())
            assert abs(an - fd) < 3e-3 * max(abs(fd), 1e-30), (which, an, fd)


@pytest.mark.parametrize("prime", [0, 1])
def test_adjoint_step_in_bands_matches_one_band(cuda_dev, prime):
    """The packed symmetric VJP in bands of tile rows (a small band budget
    splits N = 5,000 into 9 bands) against the one-band pass: same inputs,
    FP32 summation order the only difference."""
    _, ic, grav = _mods()
    lib = importlib.import_module(PKG_NAME + "._lib")
    n = 5000
    p, _, m = ic.exponential_disk(n, total_mass=5.0, seed=9)
    xm = torch.zeros((n, 4), dtype=torch.float32, device=cuda_dev)
    xm[:, :3] = torch.tensor(p, device=cuda_dev)
    xm[:, 3] = torch.tensor(m, device=cuda_dev)
    gen = torch.Generator().manual_seed(5)
    base = [torch.randn((n, 4), generator=gen).to(cuda_dev) for _ in range(3)]
    stream = torch.cuda.current_stream(cuda_dev).cuda_stream
    out = []
    for band in (1 << 30, 5 * 16 * 512 * 5):
        solver = grav.DirectGravity(n, cuda_dev)
        solver.set_sym_band(band)
        lib.call("gb_adjoint_set_variant", solver.handle, 2)
        lx, lv, la = [b.clone() for b in base]
        lm = torch.zeros(n, dtype=torch.float32, device=cuda_dev)
        l0 = solver.launch_count()
        lib.call("gb_adjoint_step", solver.handle, xm.data_ptr(), lx.data_ptr(), lv.data_ptr(), la.data_ptr(),
                 lm.data_ptr(), n, G, EPS * EPS, DT, prime, stream)
        launches = solver.launch_count() - l0
        out.append(([t.double().cpu().numpy() for t in (lx[:, :3], lv[:, :3], la[:, :3], lm)], launches))
        solver.close()
    (one, l1), (banded, l9) = out
    assert l1 == 2 and l9 == 18
    for a, b in zip(banded, one):
        assert np.all(np.isfinite(a))
        assert _rel(a, b) < 1e-5, _rel(a, b)
