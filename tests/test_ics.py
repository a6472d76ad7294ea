"""Initial-condition generators (Plummer, two-Plummer, uniform cube, serving
stream): determinism and physical sanity.  CPU only."""
from __future__ import annotations

import numpy as np


def test_plummer_deterministic_and_virialised(nb, orc):
    a = nb.ics.plummer(4096, seed=11)
    b = nb.ics.plummer(4096, seed=11)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    assert a["x"].dtype == np.float32
    assert abs(a["m"].sum() - 1.0) < 1e-5
    ke = orc.kinetic_energy(a["vx"], a["vy"], a["vz"], a["m"])
    pe = orc.potential_energy(a["x"], a["y"], a["z"], a["m"], 1.0, 0.0)
    # Plummer: PE = -3 pi G M^2 / (32 a); virial ratio 2KE/|PE| ~ 1
    assert abs(pe + 3 * np.pi / 32) < 0.03
    assert abs(2 * ke / abs(pe) - 1.0) < 0.08
    com = np.array([np.dot(a["m"], a[k]) for k in ("x", "y", "z")])
    assert np.all(np.abs(com) < 1e-5)


def test_two_plummer_geometry(nb):
    s = nb.ics.two_plummer(20000, seed=2)
    left = s["x"] < 0
    assert abs(s["m"].sum() - 1.0) < 1e-5
    assert abs(np.median(s["x"][left]) + 5) < 0.2 and abs(np.median(s["x"][~left]) - 5) < 0.2
    vrel = np.average(s["vx"][left], weights=s["m"][left]) - \
        np.average(s["vx"][~left], weights=s["m"][~left])
    assert abs(vrel - 0.3) < 0.02


def test_uniform_cube(nb):
    s = nb.ics.uniform_cube(10000, seed=3)
    for k in ("x", "y", "z"):
        assert s[k].min() >= 0 and s[k].max() < 160
    assert abs(s["m"].sum() - 1.0) < 1e-5


def test_ensemble_stream_distribution(nb):
    reqs = nb.ics.ensemble_requests(4096, seed=5, rate=10.0)
    ns = np.array([r["n"] for r in reqs])
    st = np.array([r["steps"] for r in reqs])
    arr = np.array([r["arrival"] for r in reqs])
    assert ns.min() >= 256 and ns.max() <= 65536
    # log-uniform: median near exp(mean log) = sqrt(256 * 65536) = 4096
    assert 3000 < np.median(ns) < 5600
    assert st.min() >= 100 and st.max() <= 2000
    assert np.all(np.diff(arr) >= 0) and arr[0] == 0.0
    assert abs(len(reqs) / arr[-1] - 10.0) < 1.0
