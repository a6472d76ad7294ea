"""Per-stage device times of a calculator (NBGB_FLAG_STAGE_TIMINGS): every
stage of every method is reported with its run count, the stage times add
up to no more than the evaluations' own CUDA-event time, and a reset clears
them.  The stages are what the reference's NBODY_PROFILE_SCOPE phases time
on the host (include/nbody/performance_observability.hpp:70-78), measured on
the device."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu

STAGES = {
    "direct": ["direct.forces"],
    "bh": ["barnes_hut.bounds", "barnes_hut.keys", "barnes_hut.sort", "barnes_hut.order",
           "barnes_hut.nodes", "barnes_hut.com", "barnes_hut.walk"],
    "hash": ["spatial_hash.bounds", "spatial_hash.assign", "spatial_hash.sort",
             "spatial_hash.cells", "spatial_hash.forces"],
}


@pytest.mark.parametrize("method", ["direct", "bh", "hash"])
def test_stage_times(nb, method):
    import torch

    s = nb.ics.plummer(20000, seed=31)
    calc = {"direct": nb.DirectForceCalculator, "bh": lambda: nb.BarnesHutCalculator(0.5),
            "hash": lambda: nb.SpatialHashCalculator(0.5, 0.5)}[method]()
    calc.setSofteningParameter(0.01)
    calc.set_flags(calc.params.flags | nb.FLAG_STAGE_TIMINGS)
    st = torch.cuda.current_stream()
    calc.set_stream(st.cuda_stream)
    with nb.ScopedParticleData(20000, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                       "mass": s["m"]}) as p:
        calc.computeForces(p.device)
        calc.stage_times(reset=True)  # drop the first (allocating) evaluation
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(3):
            calc.computeForces(p.device)
        e1.record(st)
        torch.cuda.synchronize()
        t = calc.stage_times()
    assert list(t) == STAGES[method]
    for name in STAGES[method]:
        ms, runs = t[name]
        assert runs == 3 and ms > 0, (name, ms, runs)
    assert sum(ms for ms, _ in t.values()) <= e0.elapsed_time(e1) * 1.02 + 0.05
    calc.stage_times(reset=True)
    assert all(v == (0.0, 0) for v in calc.stage_times().values())
    calc.close()


def test_stage_times_off_by_default(nb):
    calc = nb.DirectForceCalculator()
    s = nb.ics.plummer(1000, seed=32)
    with nb.ScopedParticleData(1000, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                      "mass": s["m"]}) as p:
        calc.computeForces(p.device)
    assert calc.stage_times() == {}
    calc.close()
