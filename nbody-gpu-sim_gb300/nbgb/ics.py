"""Seeded initial conditions for the benchmark workloads.

The reference ships uniform-box, uniform-ball and disk generators only
(src/cuda/particle_init.cu:167-234); the Plummer models used by the
benchmark configurations are generated here.  Everything is drawn from one
numpy PCG64 generator per call, so a (function, seed) pair is reproducible.
Positions and velocities are returned in float32 (the drop-in ParticleData
precision); FP64 states are initialised from exactly these values.

Plummer sphere (G = 1, total mass M, scale a), Aarseth-Henon-Wielen 1974:
  radius  r = a / sqrt(U^(-2/3) - 1), U ~ U(0,1), isotropic direction,
          no radius truncation;
  speed   v = q * v_esc(r), v_esc = sqrt(2 G M) (r^2 + a^2)^(-1/4), with q
          drawn by von Neumann rejection from g(q) = q^2 (1 - q^2)^(7/2)
          (envelope 0.1 > max g), isotropic direction;
  the centre of mass and its velocity are moved to the origin / rest, then
  the requested centre and bulk velocity are added.
"""
from __future__ import annotations

import numpy as np


def _isotropic(rng: np.random.Generator, n: int) -> np.ndarray:
    cos_t = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    sin_t = np.sqrt(np.maximum(0.0, 1.0 - cos_t * cos_t))
    return np.stack([sin_t * np.cos(phi), sin_t * np.sin(phi), cos_t], axis=1)


def _plummer_raw(rng: np.random.Generator, n: int, a: float, M: float, G: float):
    u = rng.random(n)
    while np.any(u == 0.0):
        z = u == 0.0
        u[z] = rng.random(int(z.sum()))
    r = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    pos = _isotropic(rng, n) * r[:, None]
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        x1 = rng.random(todo.size)
        x2 = rng.random(todo.size) * 0.1
        ok = x2 < x1 * x1 * (1.0 - x1 * x1) ** 3.5
        q[todo[ok]] = x1[ok]
        todo = todo[~ok]
    vesc = np.sqrt(2.0 * G * M) * (r * r + a * a) ** -0.25
    vel = _isotropic(rng, n) * (q * vesc)[:, None]
    m = np.full(n, M / n)
    pos -= np.average(pos, axis=0, weights=m)
    vel -= np.average(vel, axis=0, weights=m)
    return pos, vel, m


def _pack(pos, vel, m) -> dict[str, np.ndarray]:
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
    return dict(x=f(pos[:, 0]), y=f(pos[:, 1]), z=f(pos[:, 2]), vx=f(vel[:, 0]),
                vy=f(vel[:, 1]), vz=f(vel[:, 2]), m=f(m))


def plummer(n: int, seed: int = 1, a: float = 1.0, M: float = 1.0, G: float = 1.0,
            center=(0.0, 0.0, 0.0), bulk_velocity=(0.0, 0.0, 0.0)) -> dict[str, np.ndarray]:
    """Equal-mass Plummer sphere of n bodies (float32 arrays x..vz, m)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos, vel, m = _plummer_raw(rng, n, a, M, G)
    pos += np.asarray(center, dtype=np.float64)
    vel += np.asarray(bulk_velocity, dtype=np.float64)
    return _pack(pos, vel, m)


def two_plummer(n: int, seed: int = 2, a: float = 1.0, separation: float = 10.0,
                approach_speed: float = 0.3) -> dict[str, np.ndarray]:
    """Two equal Plummer spheres (M = 0.5 each) centred at x = -/+ separation/2,
    approaching along x at relative speed approach_speed (the Barnes-Hut
    workload: N = 1,048,576, centres x = +-5, relative speed 0.3)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n1 = n // 2
    n2 = n - n1
    p1, v1, m1 = _plummer_raw(rng, n1, a, 0.5, 1.0)
    p2, v2, m2 = _plummer_raw(rng, n2, a, 0.5, 1.0)
    half = separation / 2.0
    p1[:, 0] -= half
    p2[:, 0] += half
    v1[:, 0] += approach_speed / 2.0
    v2[:, 0] -= approach_speed / 2.0
    # each sphere has mass 0.5: per-body masses 0.5/n_k
    return _pack(np.concatenate([p1, p2]), np.concatenate([v1, v2]), np.concatenate([m1, m2]))


def uniform_cube(n: int, seed: int = 3, side: float = 160.0, total_mass: float = 1.0):
    """n equal masses (total_mass/n) uniform in [0, side)^3 at rest (the
    spatial-hash workload: N = 4,194,304, side 160)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.random((n, 3)) * side
    pos = np.minimum(pos, np.nextafter(np.float32(side), np.float32(0)))
    vel = np.zeros((n, 3))
    m = np.full(n, total_mass / n)
    return _pack(pos, vel, m)


def ensemble_requests(count: int = 4096, seed: int = 5, n_min: int = 256, n_max: int = 65536,
                      steps_min: int = 100, steps_max: int = 2000, rate: float = 1.0):
    """The serving stream: `count` Plummer clusters (a = 1, M = 1) with N
    log-uniform in [n_min, n_max], step counts uniform in [steps_min,
    steps_max], Poisson arrival times of the given rate (per second), and a
    per-request seed.  Returns a list of dicts (id, n, steps, arrival, seed)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    logn = rng.uniform(np.log(n_min), np.log(n_max), count)
    ns = np.clip(np.round(np.exp(logn)).astype(np.int64), n_min, n_max)
    steps = rng.integers(steps_min, steps_max + 1, count)
    gaps = rng.exponential(1.0 / rate, count)
    arrival = np.cumsum(gaps) - gaps[0]
    seeds = rng.integers(1, 2**31 - 1, count)
    return [dict(id=i, n=int(ns[i]), steps=int(steps[i]), arrival=float(arrival[i]),
                 seed=int(seeds[i])) for i in range(count)]
