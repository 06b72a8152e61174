"""Seeded synthetic initial conditions for the gravity workloads.

The reference's initialisers (astro/src/initialisers.rs) draw from
rand_chacha streams that are not vendored, so inputs here come from numpy's
PCG64 with fixed seeds and are handed to both the GPU path and the oracle as
the same arrays.

  cube_with_stars   uniform cube U[-0.5,0.5]^3, unit masses, solid-body spin
                    v = (-y, x, 0), plus heavy stars at given positions.
  plummer           Plummer sphere; radii from the inverse mass profile and
                    isotropic velocities from the distribution function by
                    the rejection method of Aarseth, Henon & Wielen (1974).
  ensemble_sizes    log-uniform body counts of a batched ensemble.
"""
from __future__ import annotations

import numpy as np

from .entity import from_arrays

STARS_2 = np.array([[0.2, 0.2, 0.5], [-0.2, -0.2, 0.5]])
STARS_4 = np.array([[0.1, 0.1, 0.5], [0.1, -0.1, 0.5], [-0.1, 0.1, 0.5], [-0.1, -0.1, 0.5]])


def cube_with_stars(n: int, seed: int = 1, stars: np.ndarray | None = None,
                    star_mass: float = 1e5, half: float = 0.5, spin: float = 1.0) -> np.ndarray:
    """n bodies uniform in [-half, half]^3 (mass 1, v = spin*(-y, x, 0)) followed by
    the stars (v = 0, not fixed)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.uniform(-half, half, size=(n, 3))
    vel = np.stack([-pos[:, 1], pos[:, 0], np.zeros(n)], axis=1) * spin
    mass = np.ones(n)
    if stars is not None and len(stars):
        pos = np.concatenate([pos, np.asarray(stars, dtype=np.float64)])
        vel = np.concatenate([vel, np.zeros((len(stars), 3))])
        mass = np.concatenate([mass, np.full(len(stars), star_mass)])
    ids = np.arange(len(mass), dtype=np.uint64)
    return from_arrays(pos, vel, mass, ids=ids, radius=np.full(len(mass), 0.01))


def _isotropic(rng: np.random.Generator, r: np.ndarray) -> np.ndarray:
    cos_t = rng.uniform(-1.0, 1.0, size=len(r))
    sin_t = np.sqrt(1.0 - cos_t * cos_t)
    phi = rng.uniform(0.0, 2.0 * np.pi, size=len(r))
    return np.stack([r * sin_t * np.cos(phi), r * sin_t * np.sin(phi), r * cos_t], axis=1)


def plummer(n: int, seed: int = 7, a: float = 0.1, total_mass: float = 1.0, G: float = 1.0,
            r_max: float = 100.0) -> np.ndarray:
    """Plummer sphere with scale radius a (Aarseth, Henon & Wielen 1974)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    # radius: inverse of M(<r)/M = r^3 / (r^2 + a^2)^{3/2}
    r = np.empty(n)
    filled = 0
    while filled < n:
        x = rng.uniform(0.0, 1.0, size=n - filled)
        x = x[x > 0.0]
        rr = a / np.sqrt(x ** (-2.0 / 3.0) - 1.0)
        rr = rr[rr < r_max * a]
        r[filled:filled + len(rr)] = rr
        filled += len(rr)
    pos = _isotropic(rng, r)
    # speed: q = v / v_esc with density g(q) = q^2 (1 - q^2)^{7/2}, max < 0.1
    q = np.empty(n)
    filled = 0
    while filled < n:
        m = 2 * (n - filled) + 64
        x4 = rng.uniform(0.0, 1.0, size=m)
        x5 = rng.uniform(0.0, 0.1, size=m)
        acc = x5 < x4 * x4 * (1.0 - x4 * x4) ** 3.5
        take = x4[acc][: n - filled]
        q[filled:filled + len(take)] = take
        filled += len(take)
    v_esc = np.sqrt(2.0 * G * total_mass) * (r * r + a * a) ** -0.25
    vel = _isotropic(rng, q * v_esc)
    mass = np.full(n, total_mass / n)
    # centre of mass at rest at the origin
    pos -= np.average(pos, axis=0, weights=mass)
    vel -= np.average(vel, axis=0, weights=mass)
    ids = np.arange(n, dtype=np.uint64)
    return from_arrays(pos, vel, mass, ids=ids, radius=np.full(n, 0.01))


def ensemble_sizes(count: int = 512, seed: int = 3, lo: int = 256, hi: int = 65536) -> np.ndarray:
    """N_k = floor(exp(U[ln lo, ln hi]))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi), size=count))).astype(np.int64)


# The standard workloads.
def workload_direct_small() -> np.ndarray:
    """4,096 cube bodies + 2 stars of mass 1e5 (4,098 bodies)."""
    return cube_with_stars(4096, seed=1, stars=STARS_2)


def workload_large(n: int = 1_048_576) -> np.ndarray:
    """1,048,576 cube bodies + 4 stars of mass 1e5 at (+-0.1, +-0.1, 0.5)."""
    return cube_with_stars(n, seed=1, stars=STARS_4)
