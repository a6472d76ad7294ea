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


# -- injected device-allocation failures (nbgb_selftest_fail_allocation) --------
@pytest.fixture
def fail_alloc(nb):
    f = nb.lib().nbgb_selftest_fail_allocation
    yield f
    f(0)


def _calc(nb, method):
    c = {"direct": lambda: nb.DirectForceCalculator(),
         "bh": lambda: nb.BarnesHutCalculator(0.5),
         "bhg": lambda: nb.BarnesHutCalculator(0.5, group_walk=True),
         "hash": lambda: nb.SpatialHashCalculator(2.0, 2.0)}[method]()
    c.setSofteningParameter(0.01)
    return c


def _forces(nb, calc, p):
    calc.computeForces(p.device)
    p.download()
    return [p.host[k].copy() for k in ("acc_x", "acc_y", "acc_z")]


@pytest.mark.parametrize("method", ["direct", "bh", "bhg", "hash"])
@pytest.mark.parametrize("nth", [1, 2, 4, 9])
def test_injected_oom_then_recovers(nb, fail_alloc, method, nth):
    """The nth device allocation of a calculator's first call fails: the call
    raises the reference's ResourceException, and the next call on the same
    calculator gives bit for bit what a fresh calculator gives."""
    s = nb.ics.plummer(6000, seed=9)
    arrays = {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"], "mass": s["m"]}
    with nb.ScopedParticleData(6000, arrays) as p:
        fresh = _calc(nb, method)
        want = _forces(nb, fresh, p)
        fresh.close()
        calc = _calc(nb, method)
        fail_alloc(nth)
        try:
            _forces(nb, calc, p)
            failed = False
        except nb.ResourceException as e:
            failed = True
            assert "allocation" in str(e)
            if method == "bh":  # a build that did not finish cannot be inspected
                with pytest.raises(nb.NbodyError):
                    calc.tree_stats()
        fail_alloc(0)
        if nth == 1:
            assert failed  # every first call allocates
        got = _forces(nb, calc, p)
        calc.close()
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)


def test_injected_oom_in_particle_and_system_allocation(nb, fail_alloc):
    import torch
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    s = nb.ics.plummer(3000, seed=10)
    for nth in (1, 5, 13):  # the 13 arrays of ParticleData
        fail_alloc(nth)
        with pytest.raises(nb.ResourceException):
            nb.ParticleDataManager.allocateDevice(3000)
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(0.01)
    for nth in (1, 3, 6):
        fail_alloc(nth)
        with pytest.raises(nb.ResourceException):
            nb.System(calc, s)
    fail_alloc(0)
    sysm = nb.System(calc, s)  # and now it works
    sysm.step(1e-3, 3)
    ke, pe, _ = sysm.energy()
    assert np.isfinite(ke) and pe < 0
    sysm.close()
    calc.close()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0 - (64 << 20)  # the failed attempts left nothing behind


def test_injected_oom_in_the_ensemble_then_continues(nb, fail_alloc):
    """An allocation failure inside an engine tick surfaces as an error from
    that tick; the engine then goes on, and every request completes with the
    same result as in a run without the failure."""
    from nbgb.serving import Ensemble
    reqs = [(nb.ics.plummer(n, seed=20 + n), 5) for n in (500, 3000, 12000, 20000)]

    def run(inject):
        ens = Ensemble(hbm_budget_bytes=2 << 30, direct_config=0)
        ids = {ens.submit(st, steps, 1e-3): i for i, (st, steps) in enumerate(reqs)}
        errors = 0
        if inject:
            fail_alloc(inject)
        for _ in range(200):
            try:
                if ens.tick() == (0, 0):
                    break
            except nb.NbodyError:
                errors += 1
                fail_alloc(0)
        fail_alloc(0)
        ens.synchronize()
        out = {}
        while (res := ens.poll(want_state=True)) is not None:
            out[ids[res[0]["request_id"]]] = res[1]
        ens.close()
        return out, errors

    clean, e0 = run(0)
    assert e0 == 0 and len(clean) == len(reqs)
    for nth in (1, 3, 8):
        got, errors = run(nth)
        assert errors == 1, (nth, errors)
        assert sorted(got) == sorted(clean)
        for i in clean:
            for k in ("x", "y", "z", "vx", "vy", "vz"):
                np.testing.assert_array_equal(got[i][k], clean[i][k])
