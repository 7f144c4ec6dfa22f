"""Seeded initial conditions for the engine's workloads and parity cases.

The reference's own generators (src/scenarios.cpp) differ from the workload definitions used
here (Gaussian disk profile, different defaults), so the engine ships its own. Parity never depends
on the generator: the same ``Bodies`` are given to the engine and to the CPU oracle. All columns
are built in FP64, centred on the centre of mass and rounded to float32 at the end, as the
reference's ``finish`` does (src/scenarios.cpp:52-73).

Workloads (sizes are the defaults):
  plummer(n=16384, seed=1, cut=10)       direct-summation Plummer sphere, Henon units
  disk(n=1_000_000, seed=1)              exponential disk, sech^2 vertical, core mass 1
  collision(n_each=8_000_000)            two inclined disks on a parabolic orbit
  ensemble_sizes(512)                    log-uniform cluster sizes in [1024, 131072]
  ensemble(512)                          512 Plummer clusters back to back (seeds 100-611)
Test shapes mirroring the reference tests: plummer(n, seed, cut=20), cube(n, seed).
"""
from __future__ import annotations

import math

import numpy as np

from .bodies import Bodies

HENON_A = 3.0 * math.pi / 16.0


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(int(seed)))


def _finish(pos: np.ndarray, vel: np.ndarray, m: np.ndarray, centre: bool = True) -> Bodies:
    if centre and len(m):
        M = m.sum()
        pos = pos - (m[:, None] * pos).sum(0) / M
        vel = vel - (m[:, None] * vel).sum(0) / M
    return Bodies.from_arrays(pos, vel, m)


def _unit_vectors(rng: np.random.Generator, n: int) -> np.ndarray:
    z = rng.uniform(-1.0, 1.0, n)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = 2.0 * math.pi * rng.random(n)
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)


def plummer_arrays(n: int, seed: int = 1, a: float = HENON_A, cut: float = 10.0, G: float = 1.0,
                   M: float = 1.0):
    """Plummer sphere (Aarseth, Henon & Wielen 1974) as FP64 arrays, not centred.

    Radii from the inverse cumulative mass profile, redrawn beyond ``cut * a``; speeds by von
    Neumann rejection on q^2 (1 - q^2)^3.5 (bounded by 0.1); isotropic directions.
    """
    rng = _rng(seed)
    r = np.empty(n)
    k = 0
    while k < n:
        X = rng.random(2 * (n - k) + 16)
        X = X[X > 0]
        rr = a / np.sqrt(X ** (-2.0 / 3.0) - 1.0)
        rr = rr[rr <= cut * a]
        take = min(n - k, rr.size)
        r[k:k + take] = rr[:take]
        k += take
    q = np.empty(n)
    k = 0
    while k < n:
        qq = rng.random(4 * (n - k) + 16)
        g = 0.1 * rng.random(qq.size)
        qq = qq[g < qq * qq * (1.0 - qq * qq) ** 3.5]
        take = min(n - k, qq.size)
        q[k:k + take] = qq[:take]
        k += take
    v = q * math.sqrt(2.0 * G * M / a) * (1.0 + r * r / (a * a)) ** -0.25
    pos = r[:, None] * _unit_vectors(rng, n)
    vel = v[:, None] * _unit_vectors(rng, n)
    m = np.full(n, M / n)
    return pos, vel, m


def plummer(n: int = 16384, seed: int = 1, cut: float = 10.0, a: float = HENON_A, G: float = 1.0) -> Bodies:
    pos, vel, m = plummer_arrays(n, seed, a=a, cut=cut, G=G)
    return _finish(pos, vel, m)


def cube(n: int, seed: int) -> Bodies:
    """Uniform positions and velocities in [-1, 1)^3, masses uniform in [0.5, 1.5) / n."""
    rng = _rng(seed)
    pos = rng.uniform(-1.0, 1.0, (n, 3))
    vel = rng.uniform(-1.0, 1.0, (n, 3))
    m = rng.uniform(0.5, 1.5, n) / max(n, 1)
    return _finish(pos, vel, m, centre=False)


def _disk_radii(rng: np.random.Generator, ns: int, xmax: float) -> np.ndarray:
    """Radii (in scale lengths) of a truncated exponential disk: CDF 1 - (1 + x) e^-x, inverted by
    bisection to full double precision."""
    cdf_max = 1.0 - (1.0 + xmax) * math.exp(-xmax)
    target = rng.random(ns) * cdf_max
    lo = np.zeros(ns)
    hi = np.full(ns, xmax)
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        below = 1.0 - (1.0 + mid) * np.exp(-mid) < target
        lo = np.where(below, mid, lo)
        hi = np.where(below, hi, mid)
    return 0.5 * (lo + hi)


def disk_arrays(n: int = 1_000_000, seed: int = 1, core: float = 1.0, mass: float = 1.0, rd: float = 1.0,
                rmax: float = 10.0, h: float = 0.1, dispersion: float = 0.05, G: float = 1.0):
    """Exponential disk with a central point mass, FP64 arrays, not centred.

    Surface density ~ exp(-R/rd) for R <= rmax, vertical density ~ sech^2(z/h), total disk mass
    ``mass`` over n-1 stars, a core of mass ``core`` at the origin. Circular speed from the enclosed
    mass (core plus the stars at smaller R, spherical approximation), plus Gaussian dispersion of
    ``dispersion`` times the circular speed in each component.
    """
    if n < 2:
        raise ValueError("disk needs at least 2 bodies (core + 1 star)")
    rng = _rng(seed)
    ns = n - 1
    ms = mass / ns
    R = np.sort(_disk_radii(rng, ns, rmax / rd)) * rd
    R = np.maximum(R, 1e-12 * rd)
    phi = 2.0 * math.pi * rng.random(ns)
    u = rng.random(ns)
    u = np.clip(u, 1e-15, 1.0 - 1e-15)
    z = h * np.arctanh(2.0 * u - 1.0)
    enclosed = core + ms * np.arange(1, ns + 1, dtype=np.float64)
    vc = np.sqrt(G * enclosed / R)
    sg = dispersion * vc
    cp, sp = np.cos(phi), np.sin(phi)
    noise = rng.standard_normal((ns, 3))
    pos = np.empty((n, 3))
    vel = np.empty((n, 3))
    pos[0] = 0.0
    vel[0] = 0.0
    pos[1:, 0] = R * cp
    pos[1:, 1] = R * sp
    pos[1:, 2] = z
    vel[1:, 0] = -vc * sp + sg * noise[:, 0]
    vel[1:, 1] = vc * cp + sg * noise[:, 1]
    vel[1:, 2] = sg * noise[:, 2]
    m = np.full(n, ms)
    m[0] = core
    return pos, vel, m


def disk(n: int = 1_000_000, seed: int = 1, **kw) -> Bodies:
    pos, vel, m = disk_arrays(n, seed, **kw)
    return _finish(pos, vel, m)


def _rot_x(v: np.ndarray, angle: float) -> np.ndarray:
    c, s = math.cos(angle), math.sin(angle)
    out = v.copy()
    out[:, 1] = v[:, 1] * c - v[:, 2] * s
    out[:, 2] = v[:, 1] * s + v[:, 2] * c
    return out


def collision(n_each: int = 8_000_000, seed: int = 1, incl=(45.0, 30.0), separation: float = 20.0,
              pericentre: float = 3.0, G: float = 1.0):
    """Two disks (disk() recipe) inclined by ``incl`` degrees to the orbital (x-y) plane, centres
    ``separation`` apart on a parabolic approach with the given pericentre. Returns (Bodies, n_each):
    disk 1 is ids [0, n_each)."""
    parts = []
    masses = []
    for k in range(2):
        pos, vel, m = disk_arrays(n_each, seed + k)
        M = m.sum()
        pos -= (m[:, None] * pos).sum(0) / M
        vel -= (m[:, None] * vel).sum(0) / M
        parts.append((_rot_x(pos, math.radians(incl[k])), _rot_x(vel, math.radians(incl[k])), m))
        masses.append(M)
    Mtot = masses[0] + masses[1]
    # Parabolic relative orbit: energy 0, angular momentum sqrt(2 G Mtot q), in the x-y plane.
    r0 = separation
    v0 = math.sqrt(2.0 * G * Mtot / r0)
    hmom = math.sqrt(2.0 * G * Mtot * pericentre)
    vt = hmom / r0
    vr = -math.sqrt(max(v0 * v0 - vt * vt, 0.0))
    rel_pos = np.array([r0, 0.0, 0.0])
    rel_vel = np.array([vr, vt, 0.0])
    f1 = masses[1] / Mtot
    f0 = masses[0] / Mtot
    pos = np.concatenate([parts[0][0] + f1 * rel_pos, parts[1][0] - f0 * rel_pos])
    vel = np.concatenate([parts[0][1] + f1 * rel_vel, parts[1][1] - f0 * rel_vel])
    m = np.concatenate([parts[0][2], parts[1][2]])
    return _finish(pos, vel, m), n_each


def ensemble_sizes(count: int = 512, lo: int = 1024, hi: int = 131072, seed: int = 100) -> np.ndarray:
    """Cluster sizes floor(lo * (hi/lo)^u), u uniform, one per system."""
    u = _rng(seed).random(count)
    return np.floor(lo * (hi / lo) ** u).astype(np.int64)


def ensemble_eps(n: np.ndarray, base: float = 0.01, n0: int = 16384) -> np.ndarray:
    """Per-system softening eps = base * (N / n0)^(-1/3)."""
    return base * (np.asarray(n, np.float64) / n0) ** (-1.0 / 3.0)


def ensemble(count: int = 512, lo: int = 1024, hi: int = 131072, seed0: int = 100, direct_max: int = 8192,
             theta: float = 0.5, sizes=None):
    """Independent Plummer clusters (plummer() recipe, seeds seed0 + s, each centred) back to back.

    Sizes are ensemble_sizes(count, lo, hi, seed0) unless given; softening ensemble_eps(N); direct
    summation for N <= direct_max, tree with opening angle ``theta`` above. Ids run 0..total-1.
    Returns (Bodies, counts, eps, thetas, methods) with methods 0 = direct, 1 = tree.
    """
    n = np.asarray(ensemble_sizes(count, lo, hi, seed0) if sizes is None else sizes, np.int64)
    pos, vel, m = [], [], []
    for s, ns in enumerate(n):
        p, v, ms = plummer_arrays(int(ns), seed0 + s)
        M = ms.sum()
        pos.append(p - (ms[:, None] * p).sum(0) / M)
        vel.append(v - (ms[:, None] * v).sum(0) / M)
        m.append(ms)
    b = Bodies.from_arrays(np.concatenate(pos), np.concatenate(vel), np.concatenate(m))
    methods = np.where(n <= direct_max, 0, 1).astype(np.int32)
    return b, n.astype(np.uint32), ensemble_eps(n), np.full(len(n), float(theta)), methods
