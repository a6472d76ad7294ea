"""Direct N^2 forces through the C ABI vs the oracle (GPU).

Restates tests/test_force_calculation.cpp:69-176 and adds size sweeps against
the FP64 direct sum.  Tolerances (FP32 pairwise, MUFU rsqrt):
  * reference pin (N=32 grid): |a - ref| <= 1e-3 (|ref| + 1e-3) per component;
  * compensated sum vs FP64: per-target |a - a64| / |a64| <= 2e-5 at the 99th
    percentile and <= 1e-3 worst case (targets with strong cancellation);
  * plain FP32 sum vs the oracle's FP32 reference-order sum: 1e-3 relative.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import vec_rel_err

pytestmark = pytest.mark.gpu

VARIANTS = ["scalar4", "paired8"]


def _direct(nb, s, G=1.0, eps=0.1, variant="scalar4", compensated=True):
    os.environ["NBGB_DIRECT_VARIANT"] = variant
    calc = nb.DirectForceCalculator(256)
    try:
        calc.setGravitationalConstant(G)
        calc.setSofteningParameter(eps)
        if not compensated:
            calc.set_flags(nb.FLAG_SYNC)
        n = len(s["x"])
        with nb.ScopedParticleData(n, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                       "mass": s["m"], "vel_x": s.get("vx")}) as p:
            before = {f: p.host[f].copy() for f in ("pos_x", "vel_x", "mass")}
            calc.computeForces(p.device)
            p.download()
            for f, v in before.items():  # forces must not touch pos/vel/mass
                np.testing.assert_array_equal(p.host[f], v)
            return p.host["acc_x"].copy(), p.host["acc_y"].copy(), p.host["acc_z"].copy()
    finally:
        calc.close()
        os.environ.pop("NBGB_DIRECT_VARIANT", None)


@pytest.mark.parametrize("variant", VARIANTS)
def test_single_particle_zero(nb, variant):
    # tests/test_force_calculation.cpp:69-85
    s = {k: np.array([v], np.float32) for k, v in
         (("x", 1.0), ("y", 2.0), ("z", 3.0), ("m", 5.0))}
    ax, ay, az = _direct(nb, s, 1.0, 0.1, variant)
    assert ax[0] == 0.0 and ay[0] == 0.0 and az[0] == 0.0


@pytest.mark.parametrize("variant", VARIANTS)
def test_two_body_equal_opposite(nb, variant):
    # :87-106
    s = dict(x=np.array([-0.5, 0.5], np.float32), y=np.zeros(2, np.float32),
             z=np.zeros(2, np.float32), m=np.ones(2, np.float32))
    ax, ay, az = _direct(nb, s, 1.0, 0.01, variant)
    assert abs(ax[0] + ax[1]) < 1e-5 and abs(ay[0] + ay[1]) < 1e-5
    assert ax[0] > 0


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("compensated", [True, False])
def test_grid32_matches_reference_pin(nb, orc, golden, variant, compensated):
    # :108-148, expectation from the reference pair function in ascending j
    g = golden("ref_inputs.npz")
    s = dict(x=g["grid32_x"], y=g["grid32_y"], z=g["grid32_z"], m=g["grid32_m"])
    ax, ay, az = _direct(nb, s, 1.0, 0.1, variant, compensated)
    rx, ry, rz = orc.direct_f32(s["x"], s["y"], s["z"], s["m"], 1.0, 0.1)
    for got, ref in ((ax, rx), (ay, ry), (az, rz)):
        assert np.all(np.abs(got - ref) <= 1e-3 * (np.abs(ref) + 1e-3))


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("n", [1, 2, 3, 31, 32, 33, 255, 256, 257, 1000, 1024, 4097, 20000])
def test_sizes_vs_fp64(nb, orc, variant, n):
    s = nb.ics.plummer(n, seed=100 + n)
    ax, ay, az = _direct(nb, s, 1.0, 0.01, variant)
    if n == 1:
        assert ax[0] == 0.0
        return
    bx, by, bz = orc.direct_f64(s["x"], s["y"], s["z"], s["m"], 1.0, 0.01)
    err = vec_rel_err(ax, ay, az, bx, by, bz)
    assert np.percentile(err, 99) <= 2e-5, np.percentile(err, 99)
    assert err.max() <= 1e-3, err.max()


@pytest.mark.parametrize("variant", VARIANTS)
def test_plain_sum_vs_reference_order(nb, orc, variant):
    s = nb.ics.plummer(3000, seed=7)
    ax, ay, az = _direct(nb, s, 1.0, 0.01, variant, compensated=False)
    rx, ry, rz = orc.direct_f32(s["x"], s["y"], s["z"], s["m"], 1.0, 0.01)
    err = vec_rel_err(ax, ay, az, rx, ry, rz)
    assert np.percentile(err, 99) < 1e-4 and err.max() < 1e-3


def test_gravitational_constant_and_masses(nb, orc):
    rng = np.random.default_rng(3)
    n = 777
    s = dict(x=rng.normal(size=n).astype(np.float32), y=rng.normal(size=n).astype(np.float32),
             z=rng.normal(size=n).astype(np.float32),
             m=rng.uniform(0.1, 3.0, n).astype(np.float32))
    ax, ay, az = _direct(nb, s, 6.5, 0.05)
    bx, by, bz = orc.direct_f64(s["x"], s["y"], s["z"], s["m"], 6.5, 0.05)
    assert np.percentile(vec_rel_err(ax, ay, az, bx, by, bz), 99) < 2e-5


def test_zero_softening_distinct_positions(nb, orc):
    # eps = 0 (allowed by setSofteningParameter): self term excluded
    rng = np.random.default_rng(4)
    n = 300
    s = {k: rng.uniform(-1, 1, n).astype(np.float32) for k in ("x", "y", "z")}
    s["m"] = np.full(n, 1.0 / n, np.float32)
    ax, ay, az = _direct(nb, s, 1.0, 0.0)
    assert np.all(np.isfinite(ax))
    bx, by, bz = orc.direct_f64(s["x"], s["y"], s["z"], s["m"], 1.0, 0.0)
    assert np.percentile(vec_rel_err(ax, ay, az, bx, by, bz), 99) < 1e-4


def test_hundred_body_finite_and_deterministic(nb, golden):
    # :150-176 (initSpherical radius 5, seed 42), plus bitwise determinism
    g = golden("ref_inputs.npz")
    s = {k: g[f"sph100_r5_{k}"] for k in ("x", "y", "z", "m")}
    a1 = _direct(nb, s, 1.0, 0.1)
    a2 = _direct(nb, s, 1.0, 0.1)
    for u, v in zip(a1, a2):
        assert np.all(np.isfinite(u))
        np.testing.assert_array_equal(u, v)


def test_validation_errors(nb):
    calc = nb.DirectForceCalculator(256)
    with pytest.raises(nb.ValidationException):
        calc.setGravitationalConstant(-1.0)
    with pytest.raises(nb.ValidationException):
        calc.setSofteningParameter(float("nan"))
    calc.close()
