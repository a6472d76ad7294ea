"""The headless driver nbgb_sim on the GPU: --benchmark JSON with the
reference's record schema (src/main.cpp:375-399,
performance_observability.cpp:97-139), --export / --import round trip
through the v1 checkpoint format, and the exported state equals the
device-resident system run through the Python binding on the same initial
state (same library path: bitwise)."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def app():
    sys.path.insert(0, os.path.join(ROOT, "nbody-gpu-sim_gb300"))
    from nbgb import build
    build.build()
    return build.APP_PATH


def _run(app, *args):
    r = subprocess.run([app, *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r


@pytest.mark.parametrize("method", ["direct-n2", "barnes-hut", "spatial-hash"])
def test_benchmark_json(app, tmp_path, method):
    out = tmp_path / "bench.json"
    r = _run(app, "--benchmark", "--particles", "3000", "--benchmark-steps", "5", "--method",
             method, "--benchmark-output", str(out))
    rec = json.loads(r.stdout.strip().splitlines()[-1])
    assert rec == json.loads(out.read_text())
    b = rec["benchmarks"][0]
    assert b["benchmark_name"] == "application.benchmark_mode"
    assert b["force_method"] == method.replace("-", "_")
    assert b["particle_count"] == 3000 and b["iterations"] == 5
    assert b["metrics"]["wall_time_ms"] > 0
    keys = {"dt", "gravity", "softening", "particle_count"}
    keys |= {"barnes-hut": {"theta"}, "spatial-hash": {"cell_size", "cutoff_radius"}}.get(method, set())
    assert set(b["parameters"]) == keys
    # the reference's host phase plus the device time of each force stage
    phases = {p["name"]: p for p in b["phase_timings"]}
    assert phases["simulation.update"]["samples"] == 5
    stages = {"direct-n2": ["direct.forces"],
              "barnes-hut": ["barnes_hut.bounds", "barnes_hut.keys", "barnes_hut.sort",
                             "barnes_hut.order", "barnes_hut.nodes", "barnes_hut.com",
                             "barnes_hut.walk"],
              "spatial-hash": ["spatial_hash.bounds", "spatial_hash.assign", "spatial_hash.sort",
                               "spatial_hash.cells", "spatial_hash.forces"]}[method]
    for name in stages:
        assert phases[name]["samples"] >= 5 and phases[name]["total_duration_ms"] > 0, name
    device = sum(phases[n]["total_duration_ms"] for n in stages)
    assert device <= phases["simulation.update"]["total_duration_ms"] * 1.05


def test_export_import_roundtrip_and_trajectory(app, tmp_path, nb):
    from nbgb import checkpoint
    init, mid, end = (str(tmp_path / f) for f in ("init.nbody", "mid.nbody", "end.nbody"))
    _run(app, "--benchmark", "--particles", "2000", "--benchmark-steps", "10", "--softening",
         "0.05", "--export-initial", init, "--export", mid)
    # continue from the checkpoint: parameters come from the file
    _run(app, "--benchmark", "--benchmark-steps", "10", "--import", mid, "--export", end)
    h0, s0 = checkpoint.load(init)
    h1, s1 = checkpoint.load(mid)
    h2, s2 = checkpoint.load(end)
    assert abs(h1["simulation_time"] - 10 * np.float32(0.001)) < 1e-6
    assert h2["softening"] == np.float32(0.05) and h2["particle_count"] == 2000
    # the same 10 steps through the Python binding of nbgb_system
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(0.05)
    sysm = nb.System(calc, s0)
    sysm.step(0.001, 10)
    st = sysm.read()
    sysm.close()
    calc.close()
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        np.testing.assert_array_equal(s1[k], st[k])
    assert np.abs(s2["x"] - s1["x"]).max() > 0  # it moved on after the import


def test_group_walk_option(app, tmp_path):
    r = _run(app, "--benchmark", "--particles", "20000", "--benchmark-steps", "3", "--method",
             "barnes-hut", "--bh-walk", "group")
    b = json.loads(r.stdout.strip().splitlines()[-1])["benchmarks"][0]
    assert b["parameters"]["group_walk"] == 1 and b["metrics"]["wall_time_ms"] > 0
