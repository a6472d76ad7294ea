"""Initial conditions generated on the device (nbgb_init_particles_device).

The reference's distributions (ParticleInitializer, src/cuda/particle_init.cu:
167-234) drawn from a counter-based generator: deterministic per seed and
independent of N and of the launch shape for the three reference
distributions; geometric and statistical checks per distribution (3-sigma
bounds); the Plummer sphere against its analytic half-mass radius
(a / sqrt(2^(2/3) - 1)) and virial ratio 2K/|W| = 1 (within 3 % / 5 %).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U, S, D, P = 0, 1, 2, 3
KEYS = ("pos_x", "pos_y", "pos_z", "vel_x", "vel_y", "vel_z", "acc_x", "acc_y", "acc_z", "mass")


def _gen(nb, n, dist, seed=7, **kw):
    d = nb.ParticleDataManager.allocateDevice(n)
    try:
        nb.ParticleDataManager.initDevice(d, dist, seed, **kw)
        h = nb.ParticleData.host(count=n)
        nb.ParticleDataManager.copyToHost(h, d)
        return {k: h.array(k).copy() for k in KEYS}
    finally:
        nb.ParticleDataManager.freeDevice(d)


@pytest.mark.parametrize("dist", [U, S, D, P])
def test_deterministic_per_seed(nb, dist):
    a, b = _gen(nb, 5000, dist, seed=3), _gen(nb, 5000, dist, seed=3)
    c = _gen(nb, 5000, dist, seed=4)
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k])
    assert np.any(a["pos_x"] != c["pos_x"])
    assert all(np.all(a[k] == 0) for k in ("acc_x", "acc_y", "acc_z"))


@pytest.mark.parametrize("dist", [U, S, D])
def test_prefix_independent_of_n(nb, dist):
    small, big = _gen(nb, 1000, dist), _gen(nb, 70000, dist)
    for k in KEYS:
        np.testing.assert_array_equal(small[k], big[k][:1000])


def test_uniform_box(nb):
    n = 200000
    s = _gen(nb, n, U, min_bounds=(-1, 2, 5), max_bounds=(3, 4, 6), min_mass=0.5, max_mass=1.5)
    for k, lo, hi in (("pos_x", -1, 3), ("pos_y", 2, 4), ("pos_z", 5, 6)):
        assert s[k].min() >= lo and s[k].max() <= hi
        half = (hi - lo) / 2
        assert abs(s[k].mean() - (lo + half)) < 3 * half / np.sqrt(3 * n)
    assert s["mass"].min() >= 0.5 and s["mass"].max() <= 1.5
    assert np.all(s["vel_x"] == 0)


def test_spherical_ball(nb):
    n = 200000
    s = _gen(nb, n, S, center=(1, -2, 3), radius=5.0)
    r = np.sqrt((s["pos_x"] - 1) ** 2 + (s["pos_y"] + 2) ** 2 + (s["pos_z"] - 3) ** 2)
    assert r.max() <= 5.0 * (1 + 1e-5)
    inner = np.mean(r < 2.5)  # uniform in volume: 1/8 inside half the radius
    assert abs(inner - 0.125) < 3 * np.sqrt(0.125 * 0.875 / n)
    assert np.all(s["mass"] == 1.0)


def test_disk(nb):
    n = 100000
    s = _gen(nb, n, D, radius=10.0, thickness=1.0, rotation_speed=0.5)
    r = np.hypot(s["pos_x"], s["pos_y"])
    assert r.max() <= 10.0 * (1 + 1e-5) and np.abs(s["pos_z"]).max() <= 0.5
    v2 = s["vel_x"] ** 2 + s["vel_y"] ** 2
    np.testing.assert_allclose(v2, 0.25 * r, rtol=1e-4, atol=1e-6)
    radial = (s["vel_x"] * s["pos_x"] + s["vel_y"] * s["pos_y"]) / np.maximum(r, 1e-6)
    assert np.abs(radial).max() < 1e-4
    assert np.mean(r < 5.0) == pytest.approx(0.25, abs=3 * np.sqrt(0.25 * 0.75 / n))


def test_plummer(nb):
    n = 50000
    s = _gen(nb, n, P, plummer_a=1.0, total_mass=1.0, G=1.0)
    m = s["mass"].astype(np.float64)
    assert m.sum() == pytest.approx(1.0, rel=1e-5)
    pos = np.stack([s["pos_x"], s["pos_y"], s["pos_z"]], 1).astype(np.float64)
    vel = np.stack([s["vel_x"], s["vel_y"], s["vel_z"]], 1).astype(np.float64)
    assert np.abs((m[:, None] * pos).sum(0)).max() < 1e-5
    assert np.abs((m[:, None] * vel).sum(0)).max() < 1e-5
    r = np.linalg.norm(pos, axis=1)
    r_half = np.median(r)
    assert r_half == pytest.approx(1.0 / np.sqrt(2 ** (2 / 3) - 1), rel=0.03)
    ke = 0.5 * (m * (vel ** 2).sum(1)).sum()
    d = nb.ParticleDataManager.allocateDevice(n)
    try:
        h = nb.ParticleData.host({"pos_x": s["pos_x"], "pos_y": s["pos_y"], "pos_z": s["pos_z"],
                                  "mass": s["mass"]})
        nb.ParticleDataManager.copyToDevice(d, h)
        pe = nb.Integrator().computePotentialEnergy(d, 1.0, 1e-3)
    finally:
        nb.ParticleDataManager.freeDevice(d)
    assert 2 * ke / abs(pe) == pytest.approx(1.0, rel=0.05)


def test_validation(nb):
    d = nb.ParticleDataManager.allocateDevice(10)
    try:
        with pytest.raises(nb.ValidationException):
            nb.ParticleDataManager.initDevice(d, 9)
        with pytest.raises(nb.ValidationException):
            nb.ParticleDataManager.initDevice(d, U, min_mass=2.0, max_mass=1.0)
        with pytest.raises(nb.ValidationException):
            nb.ParticleDataManager.initDevice(d, P, plummer_a=0.0)
    finally:
        nb.ParticleDataManager.freeDevice(d)
