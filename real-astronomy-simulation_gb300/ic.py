"""Seeded synthetic initial conditions for the engine's workloads.

* ``plummer`` — Plummer sphere by inverse-CDF radii and von Neumann rejection
  for speeds (Aarseth, Henon & Wielen 1974).  It consumes the numpy
  Generator in the same order as the reference sampler
  (core/ic/plummer.py:19-76), so the same seed gives the same particles.
* ``exponential_disk`` — stellar exponential disk (radial CDF inversion on
  the reference's grid, core/ic/disk.py:94-102), sech^2 vertical profile
  z = z0 atanh(2u - 1), circular speed from the spherically enclosed mass
  with a softened radius (core/ic/disk.py:46-52) plus a Gaussian dispersion
  split sigma_R, 0.5 sigma_R, 0.35 sigma_R (core/ic/disk.py:65-70).
* ``plummer_pair`` — two Plummer spheres on a parabolic approach.
* ``plummer_batch`` — many independent spheres with log-uniform sizes.

All return float64 numpy arrays (pos (N,3), vel (N,3), mass (N,)).
"""
from __future__ import annotations

import numpy as np

from .units import G as G_GALACTIC


def _directions(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform unit vectors: cos(theta) ~ U(-1, 1), phi ~ U(0, 2 pi)."""
    mu = rng.uniform(-1.0, 1.0, n)
    s = np.sqrt(1.0 - mu ** 2)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    return np.column_stack((s * np.cos(phi), s * np.sin(phi), mu))


def plummer(n: int, total_mass: float = 1.0, scale_radius: float = 1.0, seed: int = 0,
            G: float = 1.0):
    rng = np.random.default_rng(seed)
    a, M = scale_radius, total_mass
    # Enclosed-mass fraction X = r^3 / (r^2 + a^2)^{3/2}  =>  r(X).
    X = rng.random(n)
    r = a / np.sqrt(X ** (-2.0 / 3.0) - 1.0)
    pos = _directions(rng, n) * r[:, None]
    # Speed fraction q = v / v_esc from g(q) ∝ q^2 (1 - q^2)^{7/2} (max < 0.1).
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        u = rng.random(todo.size)
        w = rng.random(todo.size)
        ok = 0.1 * w < u ** 2 * (1.0 - u ** 2) ** 3.5
        q[todo[ok]] = u[ok]
        todo = todo[~ok]
    v_esc = np.sqrt(2.0 * G * M / a) * (1.0 + (r / a) ** 2) ** -0.25
    vel = _directions(rng, n) * (q * v_esc)[:, None]
    mass = np.full(n, M / n)
    return pos, vel, mass


def exponential_disk(n: int, total_mass: float = 5.0, scale_length: float = 3.0,
                     scale_height: float = 0.3, sigma_frac: float = 0.1, seed: int = 0,
                     G: float = G_GALACTIC):
    rng = np.random.default_rng(seed)
    # Radial: invert M(<R)/M = 1 - (1 + R/Rd) exp(-R/Rd) on a fixed grid.
    u = rng.random(n)
    x = np.linspace(0.0, 20.0, 100000)
    cdf = 1.0 - (1.0 + x) * np.exp(-x)
    R = np.interp(u, cdf, x) * scale_length
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    # Vertical: isothermal sheet rho ∝ sech^2(z / z0) -> z = z0 atanh(2u - 1).
    uz = rng.random(n)
    uz = np.clip(uz, 1e-12, 1.0 - 1e-12)
    z = scale_height * np.arctanh(2.0 * uz - 1.0)
    pos = np.column_stack((R * np.cos(phi), R * np.sin(phi), z))
    mass = np.full(n, total_mass / n)
    # Circular speed from the spherically enclosed mass, softened radius.
    r_sph = np.linalg.norm(pos, axis=1)
    order = np.argsort(r_sph)
    m_enc = np.empty(n)
    m_enc[order] = np.cumsum(mass[order])
    soft = 0.05 * scale_length
    v_c = np.sqrt(G * m_enc / np.sqrt(r_sph ** 2 + soft ** 2))
    Rc = np.linalg.norm(pos[:, :2], axis=1) + 1e-6
    e_R = np.column_stack((pos[:, 0] / Rc, pos[:, 1] / Rc, np.zeros(n)))
    e_phi = np.column_stack((-pos[:, 1] / Rc, pos[:, 0] / Rc, np.zeros(n)))
    sig = sigma_frac * v_c
    dR = rng.normal(0.0, sig)
    dphi = rng.normal(0.0, 0.5 * sig)
    dz = rng.normal(0.0, 0.35 * sig)
    vel = e_R * dR[:, None] + e_phi * (v_c + dphi)[:, None]
    vel[:, 2] = dz
    vel -= np.average(vel, axis=0, weights=mass)
    return pos, vel, mass


def plummer_pair(n_each: int, separation: float = 10.0, impact: float = 2.0,
                 seeds=(0, 1), G: float = 1.0):
    """Two unit Plummer spheres (a = 1, M = 1) whose centres are `separation`
    apart, approaching on a parabolic orbit (|v_rel| = sqrt(2 G (M1+M2) / d))
    with impact parameter `impact`, in the centre-of-mass frame.  Each sphere
    is first moved to its own centre of mass and rest frame."""
    p1, v1, m1 = plummer(n_each, 1.0, 1.0, seeds[0], G)
    p2, v2, m2 = plummer(n_each, 1.0, 1.0, seeds[1], G)
    p1 = p1 - np.average(p1, axis=0, weights=m1)
    v1 = v1 - np.average(v1, axis=0, weights=m1)
    p2 = p2 - np.average(p2, axis=0, weights=m2)
    v2 = v2 - np.average(v2, axis=0, weights=m2)
    d = float(separation)
    vrel = np.sqrt(2.0 * G * 2.0 / d)
    sinb = impact / d
    rel_pos = np.array([d, 0.0, 0.0])
    rel_vel = -vrel * np.array([np.sqrt(1.0 - sinb ** 2), sinb, 0.0])
    pos = np.vstack((p1 - 0.5 * rel_pos, p2 + 0.5 * rel_pos))
    vel = np.vstack((v1 - 0.5 * rel_vel, v2 + 0.5 * rel_vel))
    mass = np.concatenate((m1, m2))
    return pos, vel, mass


def batch_sizes(num_systems: int, n_lo: int = 256, n_hi: int = 16384):
    """N_s = round(exp(U(ln n_lo, ln n_hi))) with generator seed s."""
    return [int(round(np.exp(np.random.default_rng(s).uniform(np.log(n_lo), np.log(n_hi)))))
            for s in range(num_systems)]


def plummer_batch(num_systems: int, n_lo: int = 256, n_hi: int = 16384, G: float = 1.0):
    """List of (pos, vel, mass) Plummer spheres (a = 1, M = 1), system s
    sampled with seed s."""
    return [plummer(n, 1.0, 1.0, s, G) for s, n in enumerate(batch_sizes(num_systems, n_lo, n_hi))]
