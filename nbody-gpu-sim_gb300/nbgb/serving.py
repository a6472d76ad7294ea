"""Ensemble serving: many independent simulations sharing one GPU.

`Ensemble` wraps the C ABI's nbgb_ensemble (continuous batching inside the
library: admission by HBM budget, one step of every resident system per
tick, retirement).  `serve()` is the request loop used by the serving
benchmark: it submits requests at their (Poisson) arrival times, ticks the
engine, polls finished systems and records per-request latency.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .api import ParticleData, check
from ._lib import EnsembleConfig, EnsembleResult, EnsembleStats

NOT_READY = 6


def default_config(**kw) -> EnsembleConfig:
    cfg = EnsembleConfig()
    _lib.lib().nbgb_ensemble_config_default(C.byref(cfg))
    fields = {f[0] for f in cfg._fields_}
    for k, v in kw.items():
        if k not in fields:  # a misspelt option must not be dropped silently
            raise TypeError(f"unknown ensemble option {k!r}")
        setattr(cfg, k, v)
    return cfg


class Ensemble:
    def __init__(self, **cfg) -> None:
        self.cfg = default_config(**cfg)
        h = C.c_void_p()
        check(_lib.lib().nbgb_ensemble_create(C.byref(self.cfg), C.byref(h)))
        self.handle = h
        self.sizes: dict[int, int] = {}

    def submit(self, state: dict, steps: int, dt: float) -> int:
        h = ParticleData.host({"pos_x": state["x"], "pos_y": state["y"], "pos_z": state["z"],
                               "vel_x": state["vx"], "vel_y": state["vy"], "vel_z": state["vz"],
                               "mass": state["m"]})
        rid = C.c_uint64(0)
        check(_lib.lib().nbgb_ensemble_submit(self.handle, h.ptr(), steps, dt, C.byref(rid)))
        self.sizes[rid.value] = len(state["x"])
        return rid.value

    def tick(self) -> tuple[int, int]:
        r, q = C.c_int32(0), C.c_int32(0)
        check(_lib.lib().nbgb_ensemble_tick(self.handle, C.byref(r), C.byref(q)))
        return r.value, q.value

    def poll(self, want_state: bool = False, want_acc: bool = False):
        """Next finished request as (result dict, state dict or None), or None
        when nothing has finished.  The state holds the FP64 x..vz
        (want_state) and the FP32 ax, ay, az, m at the final positions
        (want_acc)."""
        res = EnsembleResult()
        f64 = None
        cap = max(self.sizes.values()) if self.sizes else 0
        if want_state and cap:
            # large enough for whichever request finishes next
            f64 = np.empty(6 * cap, np.float64)
        hout, facc = None, None
        if want_acc and cap:
            facc = np.empty((4, cap), np.float32)
            hout = _lib.ParticleDataStruct()
            hout.acc_x, hout.acc_y, hout.acc_z, hout.mass = (facc[i].ctypes.data for i in range(4))
            hout.count = cap
        st = _lib.lib().nbgb_ensemble_poll(self.handle, C.byref(res),
                                            None if hout is None else C.byref(hout),
                                            None if f64 is None else f64.ctypes.data)
        if st == NOT_READY:
            return None
        check(st)
        self.sizes.pop(res.request_id, None)
        state = None
        n = res.count
        if f64 is not None or facc is not None:
            state = {}
        if f64 is not None:
            keys = ("x", "y", "z", "vx", "vy", "vz")
            state.update({k: f64[i * n:(i + 1) * n].copy() for i, k in enumerate(keys)})
        if facc is not None:
            state.update({k: facc[i, :n].copy() for i, k in enumerate(("ax", "ay", "az", "m"))})
        return _res(res), state

    def synchronize(self) -> None:
        check(_lib.lib().nbgb_ensemble_synchronize(self.handle))

    def stream(self) -> int:
        """cudaStream_t every tick joins into (an int handle)."""
        s = C.c_void_p()
        check(_lib.lib().nbgb_ensemble_get_stream(self.handle, C.byref(s)))
        return int(s.value or 0)

    def stats(self) -> dict:
        s = EnsembleStats()
        check(_lib.lib().nbgb_ensemble_get_stats(self.handle, C.byref(s)))
        return {name: getattr(s, name) for name, _ in EnsembleStats._fields_}

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.lib().nbgb_ensemble_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _res(r: EnsembleResult) -> dict:
    return dict(request_id=r.request_id, count=r.count, steps=r.steps, method=r.method)


@dataclass
class ServeReport:
    wall_s: float = 0.0
    particle_steps: int = 0
    completed: int = 0
    latencies_s: list = field(default_factory=list)
    ticks: int = 0
    stats: dict = field(default_factory=dict)

    def percentile(self, q: float) -> float:
        return float(np.percentile(self.latencies_s, q)) if self.latencies_s else float("nan")


def serve(ens: Ensemble, requests: list[dict], make_state, dt: float = 1e-3,
          time_scale: float = 1.0, max_wall_s: float | None = None,
          on_result=None) -> ServeReport:
    """Run the request loop: request r is submitted once wall time reaches
    r['arrival'] * time_scale (all at once if time_scale == 0); the engine is
    ticked continuously; finished requests are polled and their latency
    (completion - arrival) recorded.  Returns when every request finished or
    max_wall_s elapsed."""
    rep = ServeReport()
    order = sorted(requests, key=lambda r: r["arrival"])
    arrival_of: dict[int, float] = {}
    t0 = time.perf_counter()
    nxt = 0
    pending = 0
    while True:
        now = time.perf_counter() - t0
        while nxt < len(order) and order[nxt]["arrival"] * time_scale <= now:
            r = order[nxt]
            rid = ens.submit(make_state(r), r["steps"], dt)
            arrival_of[rid] = r["arrival"] * time_scale
            nxt += 1
            pending += 1
        if pending:
            ens.tick()
            rep.ticks += 1
        while True:
            got = ens.poll()
            if got is None:
                break
            res, _ = got
            done = time.perf_counter() - t0
            rep.latencies_s.append(done - arrival_of.pop(res["request_id"]))
            rep.completed += 1
            pending -= 1
            if on_result:
                on_result(res)
        if nxt >= len(order) and pending == 0:
            break
        if max_wall_s is not None and time.perf_counter() - t0 > max_wall_s:
            break
        if not pending and nxt < len(order):
            # idle until the next arrival
            wait = order[nxt]["arrival"] * time_scale - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.01))
    ens.synchronize()
    rep.wall_s = time.perf_counter() - t0
    rep.stats = ens.stats()
    rep.particle_steps = rep.stats["particle_steps"]
    return rep
