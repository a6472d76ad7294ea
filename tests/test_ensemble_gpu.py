"""Ensemble serving through the C ABI (GPU).

* Each result is the same alone and in the mix: with a fixed direct-kernel
  configuration the final FP64 state of a system is bitwise identical
  whether it ran alone or among other systems (direct and Barnes-Hut), since
  its work decomposition does not depend on the mix.  With the autotuner on,
  the same holds within 1e-9 relative (only the direct kernel configuration
  may differ, changing summation order).
* Against the plain one-system path (nbgb_system) and the FP64 oracle: final
  positions within 2e-5, velocities within 2e-4 (100 steps, dt = 1e-3).
* Admission respects the HBM budget and the resident cap; everything
  submitted completes; memory is returned.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(nb, reqs, **cfg):
    from nbgb.serving import Ensemble
    ens = Ensemble(**cfg)
    ids = {}
    for key, (state, steps) in reqs.items():
        ids[ens.submit(state, steps, 1e-3)] = key
    out = {}
    guard = 0
    while len(out) < len(reqs):
        ens.tick()
        while True:
            got = ens.poll(want_state=True)
            if got is None:
                break
            res, st = got
            out[ids[res["request_id"]]] = (res, st)
        guard += 1
        assert guard < 10000
    stats = ens.stats()
    ens.close()
    return out, stats


def _systems(nb):
    return {
        "d300": (nb.ics.plummer(300, seed=11), 40),
        "d2000": (nb.ics.plummer(2000, seed=12), 25),
        "d5000": (nb.ics.plummer(5000, seed=13), 30),
        "b9000": (nb.ics.plummer(9000, seed=14), 20),
        "b20000": (nb.ics.plummer(20000, seed=15), 15),
    }


def test_same_alone_and_in_mix_bitwise(nb):
    sy = _systems(nb)
    mixed, _ = _run(nb, sy, direct_config=0, hbm_budget_bytes=4 << 30)
    for key in ("d2000", "b9000"):
        alone, _ = _run(nb, {key: sy[key]}, direct_config=0, hbm_budget_bytes=4 << 30)
        for k in ("x", "y", "z", "vx", "vy", "vz"):
            np.testing.assert_array_equal(alone[key][1][k], mixed[key][1][k])


def test_buckets_same_alone_and_in_mix_bitwise(nb):
    """With 8-body buckets (the Barnes-Hut workload's leaf setting) a system's
    trajectory is also the same alone and in the mix."""
    sy = _systems(nb)
    mixed, _ = _run(nb, sy, direct_config=0, hbm_budget_bytes=4 << 30, leaf_capacity=8)
    alone, _ = _run(nb, {"b20000": sy["b20000"]}, direct_config=0, hbm_budget_bytes=4 << 30,
                    leaf_capacity=8)
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        np.testing.assert_array_equal(alone["b20000"][1][k], mixed["b20000"][1][k])


def test_group_walk_same_alone_and_beside_many_bodies(nb):
    """The ensemble's groups have a fixed size, so a Barnes-Hut system's
    group walk (and trajectory) is the same alone and beside 300,000 other
    Barnes-Hut bodies (a single calculator would switch to groups of 64
    bodies from 262,144 on)."""
    sy = {"b20000": (nb.ics.plummer(20000, seed=15), 6)}
    big = {f"big{i}": (nb.ics.plummer(60000, seed=40 + i), 6) for i in range(5)}
    alone, _ = _run(nb, sy, direct_config=0, hbm_budget_bytes=4 << 30)
    mixed, _ = _run(nb, {**sy, **big}, direct_config=0, hbm_budget_bytes=4 << 30)
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        np.testing.assert_array_equal(alone["b20000"][1][k], mixed["b20000"][1][k])


def test_same_alone_and_in_mix_autotuned(nb):
    sy = _systems(nb)
    mixed, stats = _run(nb, sy, hbm_budget_bytes=4 << 30)
    alone, _ = _run(nb, {"d5000": sy["d5000"]}, hbm_budget_bytes=4 << 30)
    for k in ("x", "y", "z"):
        a, b = alone["d5000"][1][k], mixed["d5000"][1][k]
        assert np.max(np.abs(a - b)) <= 1e-9 * max(1.0, np.max(np.abs(a)))
    assert stats["retired"] == len(sy)


def test_matches_plain_system_and_fp64_oracle(nb, orc):
    s = nb.ics.plummer(1500, seed=21)
    steps = 100
    res, _ = _run(nb, {"a": (s, steps)}, direct_config=1)
    got = res["a"][1]
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(0.01)
    sysm = nb.System(calc, s)
    sysm.step(1e-3, steps)
    plain = sysm.read_f64()
    sysm.close()
    calc.close()
    st = {k: s[k].astype(np.float64) for k in ("x", "y", "z", "vx", "vy", "vz")}
    m = s["m"].astype(np.float64)
    st["ax"], st["ay"], st["az"] = orc.direct_f64(st["x"], st["y"], st["z"], m, 1.0, 0.01)
    for _ in range(steps):
        orc.vv_step_f64(st, m, 1.0, 0.01, 1e-3)
    for ref in (plain, st):
        assert max(np.abs(got[k] - ref[k]).max() for k in ("x", "y", "z")) <= 2e-5
        assert max(np.abs(got[k] - ref[k]).max() for k in ("vx", "vy", "vz")) <= 2e-4


@pytest.mark.parametrize("group_walk,leaf", [(0, 1), (1, 1), (0, 8), (1, 8)])
def test_bh_system_matches_plain_bh(nb, group_walk, leaf):
    """A Barnes-Hut system in the ensemble follows the plain one-system path
    with the same walk (one body per leaf or buckets of at most 8 bodies)."""
    s = nb.ics.plummer(12000, seed=31)
    res, _ = _run(nb, {"b": (s, 30)}, direct_config=0, group_walk=group_walk,
                  leaf_capacity=leaf)
    got = res["b"][1]
    calc = nb.BarnesHutCalculator(0.5, leaf_capacity=leaf, group_walk=bool(group_walk),
                                  group_size=64)
    calc.setSofteningParameter(0.01)
    sysm = nb.System(calc, s)
    sysm.step(1e-3, 30)
    plain = sysm.read_f64()
    sysm.close()
    calc.close()
    # same tree, walk and kick sequence: the same trajectory
    assert max(np.abs(got[k] - plain[k]).max() for k in ("x", "y", "z")) <= 1e-9


def test_budget_and_resident_cap(nb):
    from nbgb.serving import Ensemble
    # a budget that fits about two 4096-body direct systems at a time
    ens = Ensemble(hbm_budget_bytes=(1 << 20) * 4, max_resident=3, direct_config=0)
    ids = [ens.submit(nb.ics.plummer(4096, seed=40 + k), 5, 1e-3) for k in range(6)]
    peak_res, done = 0, []
    for _ in range(200):
        r, q = ens.tick()
        peak_res = max(peak_res, r)
        st = ens.stats()
        assert st["bytes_reserved"] <= 4 * (1 << 20)
        while True:
            got = ens.poll()
            if got is None:
                break
            done.append(got[0]["request_id"])
        if len(done) == len(ids):
            break
    assert sorted(done) == sorted(ids)
    assert 1 <= peak_res <= 3
    assert ens.stats()["bytes_reserved"] == 0
    ens.close()


def test_recycled_result_buffers(nb):
    """Finished requests are read back through recycled pinned buffers: a
    request that reuses the buffer of a larger one polled before it (same
    size class) reads exactly its own state, equal to a run in a fresh
    engine."""
    from nbgb.serving import Ensemble
    big, small = nb.ics.plummer(3000, seed=81), nb.ics.plummer(2500, seed=82)
    ens = Ensemble(hbm_budget_bytes=1 << 30, direct_config=0)
    got = []
    for k, state in enumerate((big, small, big)):
        rid = ens.submit(state, 7, 1e-3)
        for _ in range(100):
            ens.tick()
            if ens.stats()["retired"] > k:
                break
        ens.synchronize()  # the read-back has landed
        r = ens.poll(want_state=True, want_acc=True)
        assert r is not None and r[0]["request_id"] == rid and r[0]["count"] == len(state["x"])
        got.append(r[1])
    ens.close()
    fresh, _ = _run(nb, {"small": (small, 7)}, direct_config=0, hbm_budget_bytes=1 << 30)
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        np.testing.assert_array_equal(got[1][k], fresh["small"][1][k])
        np.testing.assert_array_equal(got[0][k], got[2][k])
    for k in ("ax", "ay", "az", "m"):
        np.testing.assert_array_equal(got[0][k], got[2][k])
    np.testing.assert_array_equal(got[1]["m"], small["m"])


def test_oversized_request_rejected(nb):
    from nbgb.serving import Ensemble
    ens = Ensemble(hbm_budget_bytes=1 << 20)
    with pytest.raises(nb.ResourceException):
        ens.submit(nb.ics.plummer(65536, seed=1), 5, 1e-3)
    ens.close()


def test_autotuner_settles(nb):
    from nbgb.serving import Ensemble
    ens = Ensemble(hbm_budget_bytes=2 << 30)
    for k in range(24):
        ens.submit(nb.ics.plummer(1024 + 256 * k, seed=60 + k), 200, 1e-3)
    for _ in range(40):
        ens.tick()
    st = ens.stats()
    assert st["tuning"] == 0 and 0 <= st["direct_config"] < 6
    assert st["direct_kernel_ms"] > 0 and st["direct_kernel_interactions"] > 0
    ens.close()


@pytest.mark.parametrize("group_walk", [0, 1])
def test_batched_bh_bitwise_vs_calculator(nb, group_walk):
    """Barnes-Hut systems of uneven N (one body, two bodies, ragged tails of
    the 32-target warp tasks, two clusters) share one batched build + walk;
    each system's final acceleration equals the single-system calculator's
    on the same FP32 positions bit for bit (reference walk and group walk)."""
    from nbgb.serving import Ensemble
    sizes = (1, 2, 33, 1500, 4097, 12000)
    ens = Ensemble(direct_max_n=0, hbm_budget_bytes=2 << 30, group_walk=group_walk)
    reqs = {}
    for i, n in enumerate(sizes):
        s = nb.ics.plummer(n, seed=70 + i) if n != 4097 else nb.ics.two_plummer(n, seed=70 + i)
        reqs[ens.submit(s, 3 + i, 1e-3)] = n
    got = {}
    for _ in range(100):
        if ens.tick() == (0, 0):
            break
    ens.synchronize()
    while (r := ens.poll(want_state=True, want_acc=True)) is not None:
        got[r[0]["request_id"]] = r[1]
    st = ens.stats()
    ens.close()
    assert len(got) == len(reqs)
    assert st["bh_interactions"] > 0 and st["direct_interactions"] == 0
    assert st["bh_walk_ms"] > 0
    for rid, s in got.items():
        pos = {k: s[k].astype(np.float32) for k in ("x", "y", "z")}
        ref = _calc_bh(nb, pos, s["m"], group_walk=group_walk)
        for k, a in zip(("ax", "ay", "az"), ref):
            np.testing.assert_array_equal(s[k], a, err_msg=f"n={reqs[rid]} {k}")


def _calc_bh(nb, pos, m, theta=0.5, eps=0.01, group_walk=0):
    # the ensemble's group walk always forms groups of up to 64 bodies
    calc = nb.BarnesHutCalculator(theta, group_walk=bool(group_walk), group_size=64)
    calc.setSofteningParameter(eps)
    n = len(m)
    with nb.ScopedParticleData(n, {"pos_x": pos["x"], "pos_y": pos["y"], "pos_z": pos["z"],
                                   "mass": m}) as p:
        calc.computeForces(p.device)
        p.download()
        acc = (p.host["acc_x"].copy(), p.host["acc_y"].copy(), p.host["acc_z"].copy())
    calc.close()
    return acc


@pytest.mark.parametrize("group_walk", [0, 1])
def test_batched_bh_many_segments_degenerate(nb, group_walk):
    """300 Barnes-Hut systems in one batched pass (a two-digit segment sort),
    among them coincident bodies (depth-32 leaves), zero-mass bodies (skipped
    subtrees) and single bodies: each equals the single-system calculator
    bit for bit."""
    from nbgb.serving import Ensemble
    ens = Ensemble(direct_max_n=0, max_resident=400, hbm_budget_bytes=2 << 30,
                   group_walk=group_walk)
    reqs = {}
    for i in range(300):
        n = 1 + (i * 7) % 40
        s = nb.ics.plummer(n, seed=100 + i)
        if i % 5 == 1 and n > 3:
            for k in ("x", "y", "z", "vx", "vy", "vz"):
                s[k][: n // 2] = s[k][0]  # a coincident half that stays coincident
        if i % 5 == 2 and n > 3:
            s["m"][::2] = 0.0  # zero-mass bodies
        reqs[ens.submit(s, 2, 1e-3)] = n
    for _ in range(20):
        if ens.tick() == (0, 0):
            break
    ens.synchronize()
    got = {}
    while (r := ens.poll(want_state=True, want_acc=True)) is not None:
        got[r[0]["request_id"]] = r[1]
    ens.close()
    assert len(got) == len(reqs)
    for rid, s in got.items():
        pos = {k: s[k].astype(np.float32) for k in ("x", "y", "z")}
        ref = _calc_bh(nb, pos, s["m"], group_walk=group_walk)
        for k, a in zip(("ax", "ay", "az"), ref):
            np.testing.assert_array_equal(s[k], a, err_msg=f"request {rid} n={reqs[rid]} {k}")
