"""Failure detection without a GPU fault.

A bounded device wait that runs out (an mbarrier nothing arrives at, waited
on through the kernels' own wait helper) returns NBGB_ERR_DEVICE_TIMEOUT with
the wait-timeout bit in the device error word; the context stays usable and
the next force evaluation is correct.  Host-side failures (validation,
oversize grids, budget rejection) are covered in the other test files.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DEVICE_TIMEOUT = 4
ERR_WAIT_TIMEOUT = 1


def test_bounded_wait_times_out_and_context_survives(nb, orc):
    bits = C.c_uint32(0)
    st = nb.lib().nbgb_selftest_wait_timeout(4096, C.byref(bits))
    assert st == DEVICE_TIMEOUT
    assert bits.value & ERR_WAIT_TIMEOUT
    assert "ran out" in nb.lib().nbgb_last_error().decode()
    # the context is still usable: a direct evaluation matches FP64
    s = nb.ics.plummer(2048, seed=5)
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(0.01)
    with nb.ScopedParticleData(2048, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                      "mass": s["m"]}) as p:
        calc.computeForces(p.device)
        p.download()
        a = np.stack([p.host["acc_x"], p.host["acc_y"], p.host["acc_z"]], 1)
    calc.close()
    ref = np.stack(orc.direct_f64(s["x"], s["y"], s["z"], s["m"], 1.0, 0.01), 1)
    err = np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert np.median(err) < 1e-6


def test_selftest_rejects_bad_limits(nb):
    bits = C.c_uint32(0)
    assert nb.lib().nbgb_selftest_wait_timeout(0, C.byref(bits)) == 1
    assert nb.lib().nbgb_selftest_wait_timeout(1 << 21, C.byref(bits)) == 1
