"""The allocation-free direct-sum entry point (GPU).

nbgb_compute_forces_direct_noalloc serves callers that may not allocate
device memory: applications that own all device memory through their own
pools (a driver allocation would bypass their accounting), and
latency-critical loops that cannot take cudaMalloc's implicit device
synchronisation.  Its scratch is static device memory shared by all calls.

This file checks, through the C ABI:
  * two calls in a row -- different sizes and data, so stale scratch from the
    first call would show -- against the FP64 direct sum of the oracle
    (per-target vector error <= 2e-5 at the 99th percentile, <= 1e-3 worst
    case, the direct-sum tolerance of tests/test_direct_gpu.py) and against
    the regular calculator entry point (nbgb_compute_forces);
  * the exact limit (65,536 bodies fill the static body array), where the
    regular planner asks for more j-splits than the static partial-sum array
    holds, so the cap is exercised;
  * that device free memory does not change across calls after a count-0
    warm-up call, and that sizes beyond the limit are rejected with a message.
It is collected last so that a run stopping at the first failure has run
every other test already.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import vec_rel_err

pytestmark = pytest.mark.gpu

MAX_BODIES = 65536
MAX_SPLITS = 8


def _entry(nb):
    fn = nb.lib().nbgb_compute_forces_direct_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_void_p]
    return fn


def _last_error(nb):
    fn = nb.lib().nbgb_last_error
    fn.restype = C.c_char_p
    return fn().decode()


def _arrays(s):
    return {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"], "mass": s["m"]}


def _calculator(nb, s, G, eps):
    calc = nb.DirectForceCalculator()
    calc.setGravitationalConstant(G)
    calc.setSofteningParameter(eps)
    with nb.ScopedParticleData(len(s["x"]), _arrays(s)) as p:
        calc.computeForces(p.device)
        p.download()
        ref = [p.host[k].copy() for k in ("acc_x", "acc_y", "acc_z")]
    calc.close()
    return ref


def _noalloc(nb, s, G, eps):
    with nb.ScopedParticleData(len(s["x"]), _arrays(s)) as p:
        st = _entry(nb)(C.addressof(p.device.struct), G, eps, None)
        assert st == 0, _last_error(nb)
        assert _last_error(nb) == ""
        p.download()
        return [p.host[k].copy() for k in ("acc_x", "acc_y", "acc_z")]


def _check(got, ref):
    err = vec_rel_err(*got, *ref)
    assert np.percentile(err, 99) <= 2e-5 and err.max() <= 1e-3, (np.percentile(err, 99),
                                                                   err.max())


def test_noalloc_matches_oracle_and_calculator_on_two_calls(nb, orc):
    cases = [(nb.ics.plummer(40000, seed=71), 1.0, 0.01), (nb.ics.plummer(3001, seed=72), 2.5, 0.05)]
    for s, G, eps in cases:
        got = _noalloc(nb, s, G, eps)
        _check(got, orc.direct_f64(s["x"], s["y"], s["z"], s["m"], G, eps))
        _check(got, _calculator(nb, s, G, eps))


def test_noalloc_at_the_limit_caps_the_splits(nb, orc):
    fn = nb.lib().nbgb_selftest_noalloc_plan
    fn.restype = C.c_int
    fn.argtypes = [C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    planned, used = C.c_int32(0), C.c_int32(0)
    assert fn(MAX_BODIES, C.byref(planned), C.byref(used)) == 0, _last_error(nb)
    assert 1 <= used.value <= MAX_SPLITS
    assert used.value == min(planned.value, used.value)
    s = nb.ics.plummer(MAX_BODIES, seed=74)
    tgt = np.random.default_rng(5).choice(MAX_BODIES, 4096, replace=False)
    for _ in range(2):  # two calls in a row on the full scratch
        got = _noalloc(nb, s, 1.0, 0.01)
        ref = orc.direct_f64(s["x"], s["y"], s["z"], s["m"], 1.0, 0.01, targets=tgt)
        _check([g[tgt] for g in got], ref)


def test_noalloc_allocates_nothing_after_warmup(nb):
    import torch

    s = nb.ics.plummer(20000, seed=75)
    with nb.ScopedParticleData(len(s["x"]), _arrays(s)) as p:
        empty = nb.ParticleData()  # count 0: only resolves (and reserves) the scratch
        assert _entry(nb)(C.addressof(empty.struct), 1.0, 0.01, None) == 0, _last_error(nb)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(3):
            assert _entry(nb)(C.addressof(p.device.struct), 1.0, 0.01, None) == 0
        free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_sizes_beyond_the_limit(nb):
    s = nb.ics.plummer(MAX_BODIES + 1, seed=73)
    with nb.ScopedParticleData(MAX_BODIES + 1, _arrays(s)) as p:
        assert _entry(nb)(C.addressof(p.device.struct), 1.0, 0.01, None) == 1  # INVALID_ARG
        assert "65536" in _last_error(nb)
