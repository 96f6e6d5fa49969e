"""Seeded synthetic scenes in the reference Particle layout (32 B per body).

The workloads are synthetic, generated from a stated seed with numpy's PCG64:
  * uniform   -- positions uniform in [0, 1)^3, zero velocities;
  * plummer   -- Plummer sphere (scale radius a, centre c, truncated at r_max),
                 positions by inverting the enclosed-mass profile and
                 isotropic velocities from the Plummer distribution function
                 by the rejection method of Aarseth, Henon & Wielen (1974,
                 A&A 37, 183), for G = 1 and the sphere's mass;
  * clusters  -- a mixture of k Plummer spheres with equal body counts,
                 scale radii log-uniform in [a_min, a_max], centres uniform in
                 a box, Gaussian bulk velocities plus internal Plummer
                 velocities.
Masses are equal (1/N); the solver takes them from the body count.
"""
from __future__ import annotations

import numpy as np

from . import PARTICLE_DTYPE


def _empty(n: int) -> np.ndarray:
    out = np.zeros(n, PARTICLE_DTYPE)
    return out


def _unit_vectors(rng: np.random.Generator, n: int) -> np.ndarray:
    z = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)


def uniform(n: int, seed: int = 1) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    out = _empty(n)
    out["pos"] = rng.random((n, 3), dtype=np.float32)
    return out


def _plummer_offsets(rng: np.random.Generator, n: int, a: float, r_max: float, mass: float):
    # Enclosed mass fraction M(<r)/M = r^3 / (r^2 + a^2)^(3/2); truncate at r_max.
    m_max = r_max ** 3 / (r_max ** 2 + a ** 2) ** 1.5
    m = rng.uniform(0.0, m_max, n)
    m = np.maximum(m, 1e-12)
    r = a / np.sqrt(m ** (-2.0 / 3.0) - 1.0)
    pos = r[:, None] * _unit_vectors(rng, n)
    # Speed: v = q * v_esc, q ~ q^2 (1 - q^2)^(7/2) by rejection (max of g ~ 0.092).
    q = np.empty(n)
    todo = np.arange(n)
    while len(todo):
        x = rng.uniform(0.0, 1.0, len(todo))
        y = rng.uniform(0.0, 0.1, len(todo))
        ok = y < x * x * (1.0 - x * x) ** 3.5
        q[todo[ok]] = x[ok]
        todo = todo[~ok]
    v_esc = np.sqrt(2.0 * mass / a) * (1.0 + (r / a) ** 2) ** -0.25
    vel = (q * v_esc)[:, None] * _unit_vectors(rng, n)
    return pos, vel


def plummer(n: int, seed: int = 2, a: float = 0.1, center=(0.5, 0.5, 0.5), r_max: float = 0.5,
            mass: float = 1.0) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    pos, vel = _plummer_offsets(rng, n, a, r_max, mass)
    out = _empty(n)
    out["pos"] = (pos + np.asarray(center)[None, :]).astype(np.float32)
    out["vel"] = vel.astype(np.float32)
    return out


def clusters(n: int, k: int = 8, seed: int = 3, a_min: float = 0.02, a_max: float = 0.1,
             box=(0.2, 0.8), sigma_bulk: float = 0.05, truncate: float = 5.0) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.full(k, n // k)
    counts[: n - counts.sum()] += 1
    out = _empty(n)
    start = 0
    for c in range(k):
        a = float(np.exp(rng.uniform(np.log(a_min), np.log(a_max))))
        centre = rng.uniform(box[0], box[1], 3)
        bulk = rng.normal(0.0, sigma_bulk, 3)
        pos, vel = _plummer_offsets(rng, int(counts[c]), a, truncate * a, 1.0 / k)
        sl = slice(start, start + int(counts[c]))
        out["pos"][sl] = (pos + centre[None, :]).astype(np.float32)
        out["vel"][sl] = (vel + bulk[None, :]).astype(np.float32)
        start += int(counts[c])
    # Interleave clusters so the caller's order carries no spatial structure.
    perm = rng.permutation(n)
    return out[perm]


def make(kind: str, n: int, seed: int) -> np.ndarray:
    if kind == "uniform":
        return uniform(n, seed)
    if kind == "plummer":
        return plummer(n, seed)
    if kind == "clusters":
        return clusters(n, 8, seed)
    if kind == "clusters4":
        return clusters(n, 4, seed, a_min=0.1, a_max=0.1)
    raise ValueError(kind)
