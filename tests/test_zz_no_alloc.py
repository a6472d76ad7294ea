"""The allocation-free direct-sum entry point (GPU).

nbgb_compute_forces_direct_noalloc serves callers that may not allocate
device memory (applications that own all device memory through their own
pools, latency-critical loops that cannot take cudaMalloc's implicit device
synchronisation).  Its scratch is static device memory shared by all calls.
This file checks, through the C ABI, that two calls in a row -- different
sizes and data, so stale scratch from the first call would show -- give the
same accelerations as the regular calculator entry point (nbgb_compute_forces)
within the direct-sum tolerance used in tests/test_direct_gpu.py, and that
sizes beyond the static limit are rejected.  It is collected last so that a
run stopping at the first failure has run every other test already.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import vec_rel_err

pytestmark = pytest.mark.gpu

MAX_BODIES = 65536


def _entry(nb):
    fn = nb.lib().nbgb_compute_forces_direct_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_void_p]
    return fn


def _forces_both(nb, s, G, eps):
    n = len(s["x"])
    arrays = {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"], "mass": s["m"]}
    calc = nb.DirectForceCalculator()
    calc.setGravitationalConstant(G)
    calc.setSofteningParameter(eps)
    with nb.ScopedParticleData(n, arrays) as p:
        calc.computeForces(p.device)
        p.download()
        ref = [p.host[k].copy() for k in ("acc_x", "acc_y", "acc_z")]
    calc.close()
    with nb.ScopedParticleData(n, arrays) as p:
        st = _entry(nb)(C.addressof(p.device.struct), G, eps, None)
        assert st == 0, nb.lib().nbgb_last_error()
        p.download()
        got = [p.host[k].copy() for k in ("acc_x", "acc_y", "acc_z")]
    return got, ref


def test_noalloc_matches_calculator_on_two_calls(nb):
    cases = [(nb.ics.plummer(40000, seed=71), 1.0, 0.01), (nb.ics.plummer(3001, seed=72), 2.5, 0.05)]
    for s, G, eps in cases:
        got, ref = _forces_both(nb, s, G, eps)
        err = vec_rel_err(*got, *ref)
        assert np.percentile(err, 99) <= 2e-5 and err.max() <= 1e-3, err.max()


def test_noalloc_rejects_sizes_beyond_the_limit(nb):
    s = nb.ics.plummer(MAX_BODIES + 1, seed=73)
    with nb.ScopedParticleData(MAX_BODIES + 1, {"pos_x": s["x"], "pos_y": s["y"],
                                                "pos_z": s["z"], "mass": s["m"]}) as p:
        assert _entry(nb)(C.addressof(p.device.struct), 1.0, 0.01, None) == 1  # INVALID_ARG
