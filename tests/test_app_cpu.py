"""The headless driver nbgb_sim: command line and initial conditions (CPU).

Option parsing and validation messages follow the reference application
(src/core/app_cli.cpp:52-140); the default initial state (initSpherical,
radius 10, seed 42) equals the reference's own output (golden sph100_r10,
made by the reference's ParticleInitializer) bit for bit on x86-64.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def app():
    sys.path.insert(0, os.path.join(ROOT, "nbody-gpu-sim_gb300"))
    from nbgb import build
    build.build()
    return build.APP_PATH


def _run(app, *args):
    return subprocess.run([app, *args], capture_output=True, text=True, timeout=120)


def test_help(app):
    r = _run(app, "--help")
    assert r.returncode == 0 and "--benchmark-output P" in r.stdout and "--bh-walk" in r.stdout


@pytest.mark.parametrize("args,msg", [
    (("--method", "foo"), "Validation Error: Unsupported force method: foo"),
    (("--particles",), "Validation Error: Missing value for --particles"),
    (("--particles", "abc"), "Validation Error: Invalid numeric value for --particles: abc"),
    (("--frobnicate",), "Validation Error: Unknown argument: --frobnicate"),
    (("--dt", "0"), "Validation Error: Time step must be positive"),
    (("--dt", "2"), "Validation Error: Time step is too large (max 1.0)"),
    (("--softening", "0"), "Validation Error: Softening parameter must be positive"),
    (("--theta", "3"), "Validation Error: Barnes-Hut theta must be between 0 and 2"),
    (("--particles", "0"), "Validation Error: Particle count must be greater than 0"),
    (("--benchmark-steps", "0"), "Validation Error: Benchmark steps must be greater than zero"),
    (("--bh-walk", "sideways"), "Validation Error: Unsupported Barnes-Hut walk: sideways"),
])
def test_cli_validation(app, args, msg):
    r = _run(app, *args)
    assert r.returncode == 1
    assert msg in r.stderr


def test_interactive_mode_unavailable(app):
    r = _run(app, "--particles", "10")
    assert r.returncode == 1 and "--benchmark" in r.stderr


def test_initial_state_matches_reference(app, tmp_path, golden):
    from nbgb import checkpoint
    f = tmp_path / "init.nbody"
    _run(app, "--benchmark", "--particles", "100", "--benchmark-steps", "1",
         "--export-initial", str(f))  # stepping needs a GPU; the initial state is written first
    hdr, arr = checkpoint.load(str(f))
    assert hdr["particle_count"] == 100 and hdr["force_method"] == 0
    g = golden("ref_inputs.npz")
    for k in ("x", "y", "z", "vx", "vy", "vz", "m"):
        if platform.machine() in ("x86_64", "AMD64"):
            np.testing.assert_array_equal(arr[k], g[f"sph100_r10_{k}"])
        else:  # another libm: within a few ulp
            np.testing.assert_allclose(arr[k], g[f"sph100_r10_{k}"], rtol=1e-6, atol=1e-6)


def test_import_rejects_bad_file(app, tmp_path):
    f = tmp_path / "bad.nbody"
    f.write_bytes(b"NOPE" + bytes(60))
    r = _run(app, "--benchmark", "--import", str(f))
    assert r.returncode == 1 and "Invalid file format: wrong magic number" in r.stderr
