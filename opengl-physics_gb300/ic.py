"""Seeded synthetic initial conditions for the benchmark workloads.

These stand in for the reference's scenario generators
(projects/nbody_core/include/ngrav/ic/Plummer.hpp, src/Scenarios.cpp), with
the sampling rules of the benchmark specification rather than the
reference's own (which clips r at 20a and uses std::mt19937):

* ``plummer``: radius by inverse CDF r = a / sqrt(u^(-2/3) - 1), redrawn until
  r < 20a; isotropic directions; speed q * v_esc with q drawn by von Neumann
  rejection on g(q) = q^2 (1 - q^2)^3.5 (envelope 0.1, as Plummer.hpp:64-69);
  isotropic velocity directions; equal masses M/N; shifted to the
  centre-of-mass frame; rounded to FP32.
* ``uniform_ball``: positions uniform in the unit ball by rejection from the
  cube, zero velocity (the cold-collapse workload).

All arrays are returned as float32 (the workload's storage precision).
Generation uses numpy's PCG64 stream for the given seed.
"""
from __future__ import annotations

import numpy as np


def _isotropic(rng, n):
    cos_t = 2.0 * rng.random(n) - 1.0
    sin_t = np.sqrt(np.maximum(0.0, 1.0 - cos_t * cos_t))
    phi = 2.0 * np.pi * rng.random(n)
    return sin_t * np.cos(phi), sin_t * np.sin(phi), cos_t


def plummer(n: int, seed: int = 0, total_mass: float = 1.0, a: float = 1.0, G: float = 1.0, rmax: float = 20.0):
    """Plummer sphere; returns (x, y, z, vx, vy, vz, m) as float32 arrays."""
    rng = np.random.default_rng(seed)
    r = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        u = rng.random(todo.size)
        with np.errstate(divide="ignore", invalid="ignore"):
            rr = 1.0 / np.sqrt(np.power(u, -2.0 / 3.0) - 1.0)
        ok = np.isfinite(rr) & (rr < rmax)
        r[todo[ok]] = rr[ok]
        todo = todo[~ok]
    dx, dy, dz = _isotropic(rng, n)
    x, y, z = dx * r * a, dy * r * a, dz * r * a
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        qq = rng.random(todo.size)
        g = 0.1 * rng.random(todo.size)
        ok = g <= qq * qq * np.power(1.0 - qq * qq, 3.5)
        q[todo[ok]] = qq[ok]
        todo = todo[~ok]
    vesc = np.sqrt(2.0) * np.power(1.0 + r * r, -0.25)
    speed = q * vesc * np.sqrt(G * total_mass / a)
    ux, uy, uz = _isotropic(rng, n)
    vx, vy, vz = ux * speed, uy * speed, uz * speed
    m = np.full(n, total_mass / n)
    for arr in (x, y, z):
        arr -= np.sum(m * arr) / np.sum(m)
    for arr in (vx, vy, vz):
        arr -= np.sum(m * arr) / np.sum(m)
    return tuple(np.asarray(v, dtype=np.float32) for v in (x, y, z, vx, vy, vz, m))


def hernquist_sigma2(r, M=1.0, a=1.0, G=1.0):
    """Isotropic Jeans velocity dispersion of an isolated Hernquist sphere
    (Hernquist 1990, ApJ 356, 359, eq. 10)."""
    x = r / a
    t = 12.0 * x * (1.0 + x) ** 3 * np.log((1.0 + x) / x) - x / (1.0 + x) * (25.0 + 52.0 * x + 42.0 * x * x +
                                                                               12.0 * x ** 3)
    return np.maximum(G * M / (12.0 * a) * t, 0.0)


def galaxy(n_halo: int = 3774874, n_disk: int = 419430, seed: int = 3, G: float = 1.0):
    """Two-component galaxy: Hernquist halo (M 0.9, a 1, r < 30, isotropic
    Gaussian velocities with the local Jeans dispersion) + exponential disk
    (M 0.1, R_d 0.2, R < 2, sech^2 vertical profile z0 0.02, circular speed of
    the enclosed mass plus 10% Gaussian dispersion per component)."""
    rng = np.random.default_rng(seed)
    Mh, a, rcut = 0.9, 1.0, 30.0
    r = np.empty(n_halo)
    todo = np.arange(n_halo)
    while todo.size:
        s = np.sqrt(rng.random(todo.size))
        with np.errstate(divide="ignore"):
            rr = a * s / (1.0 - s)
        ok = np.isfinite(rr) & (rr < rcut) & (rr > 0.0)
        r[todo[ok]] = rr[ok]
        todo = todo[~ok]
    ux, uy, uz = _isotropic(rng, n_halo)
    hx, hy, hz = ux * r, uy * r, uz * r
    sig = np.sqrt(hernquist_sigma2(r, Mh, a, G))
    hv = rng.standard_normal((3, n_halo)) * sig
    # disk
    Md, Rd, Rmax, z0 = 0.1, 0.2, 2.0, 0.02
    R = np.empty(n_disk)
    todo = np.arange(n_disk)
    while todo.size:
        rr = rng.gamma(2.0, Rd, todo.size)
        ok = rr < Rmax
        R[todo[ok]] = rr[ok]
        todo = todo[~ok]
    phi = 2.0 * np.pi * rng.random(n_disk)
    zz = z0 * np.arctanh(np.clip(2.0 * rng.random(n_disk) - 1.0, -1 + 1e-15, 1 - 1e-15))
    dx, dy = R * np.cos(phi), R * np.sin(phi)
    norm = 1.0 - (1.0 + Rmax / Rd) * np.exp(-Rmax / Rd)
    m_disk_in = Md * (1.0 - (1.0 + R / Rd) * np.exp(-R / Rd)) / norm
    m_halo_in = Mh * R * R / (R + a) ** 2
    vc = np.sqrt(G * (m_disk_in + m_halo_in) / np.maximum(R, 1e-12))
    dv = rng.standard_normal((3, n_disk)) * (0.1 * vc)
    dvx, dvy, dvz = -vc * np.sin(phi) + dv[0], vc * np.cos(phi) + dv[1], dv[2]
    x = np.concatenate([hx, dx])
    y = np.concatenate([hy, dy])
    z = np.concatenate([hz, zz])
    vx = np.concatenate([hv[0], dvx])
    vy = np.concatenate([hv[1], dvy])
    vz = np.concatenate([hv[2], dvz])
    m = np.concatenate([np.full(n_halo, Mh / n_halo), np.full(n_disk, Md / n_disk)])
    mt = m.sum()
    for arr in (x, y, z, vx, vy, vz):
        arr -= np.sum(m * arr) / mt
    return tuple(np.asarray(v, dtype=np.float32) for v in (x, y, z, vx, vy, vz, m))


def ensemble_sizes(nsys: int = 512, lo: int = 1024, hi: int = 65536, seed: int = 0):
    """Per-system particle counts, log-uniform in [lo, hi], rounded."""
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), nsys))).astype(np.int64)


def ensemble(nsys: int = 512, lo: int = 1024, hi: int = 65536, size_seed: int = 0):
    """Ensemble of Plummer spheres (system i: seed i, N_i log-uniform in
    [lo, hi]), concatenated; returns (x, y, z, vx, vy, vz, m), offsets."""
    sizes = ensemble_sizes(nsys, lo, hi, size_seed)
    parts = [plummer(int(n), seed=i) for i, n in enumerate(sizes)]
    arrs = tuple(np.concatenate([p[c] for p in parts]) for c in range(7))
    return arrs, np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)


def uniform_ball(n: int, seed: int = 4, radius: float = 1.0, total_mass: float = 1.0):
    """Uniform-density ball by rejection from the cube, at rest."""
    rng = np.random.default_rng(seed)
    pts = np.empty((n, 3))
    filled = 0
    while filled < n:
        c = rng.random((max(1024, int(2.0 * (n - filled))), 3)) * 2.0 - 1.0
        c = c[np.einsum("ij,ij->i", c, c) < 1.0]
        take = min(len(c), n - filled)
        pts[filled:filled + take] = c[:take]
        filled += take
    pts *= radius
    z = np.zeros(n, dtype=np.float32)
    m = np.full(n, total_mass / n, dtype=np.float32)
    return (pts[:, 0].astype(np.float32), pts[:, 1].astype(np.float32), pts[:, 2].astype(np.float32), z, z.copy(),
            z.copy(), m)
