"""Host logic of the serving request loop (CPU, with a fake engine that
mimics the ensemble's admission and retirement rules)."""
from __future__ import annotations

import numpy as np
import pytest


class FakeEngine:
    """Admits up to `cap` systems FIFO, one step per tick, retires at steps."""

    def __init__(self, cap=3, tick_s=0.0):
        self.cap = cap
        self.queue, self.resident, self.done = [], [], []
        self.next_id = 1
        self.ticks = 0
        self.ps = 0
        self.tick_s = tick_s

    def submit(self, state, steps, dt):
        rid = self.next_id
        self.next_id += 1
        self.queue.append([rid, len(state["x"]), steps])
        return rid

    def tick(self):
        while self.queue and len(self.resident) < self.cap:
            self.resident.append(self.queue.pop(0))
        for r in self.resident:
            r[2] -= 1
            self.ps += r[1]
        self.done += [r for r in self.resident if r[2] == 0]
        self.resident = [r for r in self.resident if r[2] > 0]
        self.ticks += 1
        if self.tick_s:
            import time
            time.sleep(self.tick_s)
        return len(self.resident), len(self.queue)

    def poll(self, want_state=False):
        if not self.done:
            return None
        r = self.done.pop(0)
        return dict(request_id=r[0], count=r[1], steps=0, method=0), None

    def synchronize(self):
        pass

    def stats(self):
        return dict(particle_steps=self.ps, ticks=self.ticks)


def test_serve_completes_everything_in_order_of_arrival(nb):
    from nbgb.serving import serve
    reqs = [dict(id=i, n=10 + i, steps=3 + (i % 4), arrival=0.0, seed=i) for i in range(12)]
    eng = FakeEngine(cap=4)
    rep = serve(eng, reqs, lambda r: {"x": np.zeros(r["n"], np.float32)}, time_scale=0.0)
    assert rep.completed == 12
    assert rep.particle_steps == sum(r["n"] * r["steps"] for r in reqs)
    assert len(rep.latencies_s) == 12 and min(rep.latencies_s) >= 0.0
    assert rep.percentile(99) >= rep.percentile(50)


def test_serve_respects_arrival_times(nb):
    from nbgb.serving import serve
    reqs = [dict(id=i, n=5, steps=2, arrival=0.05 * i, seed=i) for i in range(5)]
    eng = FakeEngine(cap=2, tick_s=0.001)
    rep = serve(eng, reqs, lambda r: {"x": np.zeros(r["n"], np.float32)}, time_scale=1.0)
    assert rep.completed == 5
    assert rep.wall_s >= 0.2  # the last request arrives at 0.2 s
    assert max(rep.latencies_s) < 0.2  # each is served soon after it arrives


def test_serve_stops_at_wall_limit(nb):
    from nbgb.serving import serve
    reqs = [dict(id=i, n=5, steps=10**6, arrival=0.0, seed=i) for i in range(2)]
    rep = serve(FakeEngine(cap=2), reqs, lambda r: {"x": np.zeros(5, np.float32)},
                time_scale=0.0, max_wall_s=0.2)
    assert rep.completed == 0 and rep.ticks > 0


def test_ensemble_config_rejects_unknown_options(nb):
    from nbgb.serving import default_config
    cfg = default_config(group_walk=0, theta=0.7)
    assert cfg.group_walk == 0 and abs(cfg.theta - 0.7) < 1e-7
    with pytest.raises(TypeError, match="grup_walk"):
        default_config(grup_walk=0)
