"""The drop-in adapter's own logic at run time (CPU; needs the reference
sources, skipped without).

nbody-gpu-sim_gb300/adapter/nbody_adapter.cpp defines the reference's
classes over the C ABI.  Here it runs against a fake of that ABI
(tests/adapter_runtime/fake_nbgb.c: every call logged, failures planted)
driven by tests/adapter_runtime/driver.cpp, so the adapter's handle
bookkeeping, its mapping of status codes to the reference's exception types
(include/nbody/error_handling.hpp) and the call sequence of
Integrator::integrate (src/cuda/integrator.cu:175-189 semantics, FP64 state
in the library) are checked without a GPU.  The real library behind the same
calls is covered by the GPU tests through ctypes.
"""
from __future__ import annotations

import subprocess

import pytest


@pytest.fixture(scope="module")
def lines():
    from oracle import build as obuild
    exe = obuild.link_adapter_runtime()
    if exe is None:
        pytest.skip("reference sources not present")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {}
    for ln in r.stdout.splitlines():
        k, _, v = ln.partition(": ")
        out[k] = v.strip()
    return out


def test_one_calculator_per_object_released_with_it(lines):
    # create (method 1 = Barnes-Hut, handle 1), reuse with new parameters,
    # destroy; a new object in the same storage gets a new calculator
    # (the reference tree flag: the reference's own tree wherever it differs)
    assert lines["bh_lifecycle"] == ("create:1:1:reftree compute:1:4 set_params:1 compute:1:4 "
                                     "destroy:1 create:1:2:reftree compute:2:4 destroy:2")


def test_tree_inspection_uses_the_reference_tree(lines):
    # BarnesHutTree (the class the reference's tests inspect) asks for the
    # reference's own insertion tree (NBGB_FLAG_REFERENCE_TREE)
    assert lines["tree_build"] == "create:1:3:reftree destroy:3"


def test_direct_calculators_share_one_library_calculator(lines):
    assert lines["direct_shared"] == "create:0:4 compute:4:4 set_params:4 compute:4:4"


def test_status_codes_map_to_reference_exceptions(lines):
    assert lines["invalid_arg"] == \
        "ValidationException|Validation Error: Particle count must be greater than 0"
    assert lines["oom"].startswith("ResourceException|out of device memory")
    assert lines["overflow"] == "runtime_error|Spatial hash grid exceeds 1e8 cells"
    assert lines["timeout"] == "CudaException|a bounded device wait ran out of iterations"
    assert lines["no_device"] == "CudaException|no CUDA device"
    assert lines["recovered"] == "no exception"


def test_integrate_keeps_fp64_state_and_releases_it(lines):
    # kick-drift, the calculator (created at its first use), kick
    assert lines["integrate_fp64"] == ("kick_drift:4 create:1:6:reftree compute:6:4 kick:4 "
                                       "kick_drift:4 set_params:6 compute:6:4 kick:4")
    # NBGB_FP32_VERLET=1: the reference's three FP32 kernels around the forces
    assert lines["integrate_fp32"] == ("store_old update_positions set_params:6 compute:6:4 "
                                       "update_velocities")
    assert lines["energy"] == "-0.500"
    assert lines["integrate_invalid"] == \
        "ValidationException|Validation Error: Time step must be positive and finite"
    # the calculator goes first (declared last), then the integrator releases
    # the FP64 state of the ParticleData it integrated
    assert lines["integrator_released"] == "destroy:6 release:4"
