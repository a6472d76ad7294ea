"""Drop-in at link level (CPU; needs the reference sources, skipped without).

The reference's unchanged benchmark driver (benchmarks/benchmark_main.cpp),
ParticleSystem, utilities and example_basic are compiled from the reference
sources and linked with the hot-path classes of
nbody-gpu-sim_gb300/adapter/nbody_adapter.cpp and libnbgb.so instead of the
reference's src/cuda/force_*.cu and integrator.cu.  No kernel runs here.
"""
from __future__ import annotations

import subprocess

import pytest


@pytest.fixture(scope="module")
def apps(nb):
    from oracle import build as obuild
    if not obuild.reference_available():
        pytest.skip("reference sources not present")
    import os
    return obuild.link_reference_apps(os.path.dirname(nb.lib_path()))


def test_reference_apps_link_against_the_library(apps):
    for exe in apps.values():
        undef = subprocess.run(["nm", "-u", exe], capture_output=True, text=True, check=True).stdout
        assert "nbgb_compute_forces" in undef  # the force path comes from libnbgb
        ldd = subprocess.run(["ldd", exe], capture_output=True, text=True).stdout
        assert "libnbgb.so" in ldd


def test_reference_benchmark_driver_runs_its_host_only_benchmark(apps):
    r = subprocess.run([apps["nbody_benchmarks"], "--list"], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 0 and "force.barnes_hut" in r.stdout
    r = subprocess.run([apps["nbody_benchmarks"], "--benchmark", "serialization.round_trip",
                        "--particle-count", "1000", "--iterations", "2"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and '"benchmark_name":"serialization.round_trip"' in r.stdout
