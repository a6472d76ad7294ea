"""Precision study of the direct path: FP32 plain vs FP32 compensated with
FP64 state vs full FP64, on one Plummer sphere.

* Force error: accelerations of `samples` seeded targets against the FP64
  direct sum on the same FP32 positions (nbgb_direct_f64), as the vector
  relative error |a - a64| / |a64|; median and p99.
* Energy drift: |E(T) - E(0)| / |E(0)| after `steps` steps of dt, energies
  from each variant's state by the FP64 energy kernel (PE in FP64 from the
  positions; FP32 states are exact in FP64).

Variants:
  fp32        the reference's scheme: FP32 state and the drop-in Velocity
              Verlet (nbgb_integrate), FP32 forces with one running FP32
              accumulator per target (NBGB_FLAG_COMPENSATED cleared);
  fp32c_fp64  FP32 forces with per-tile compensated accumulation, FP64 x, v
              (nbgb_system);
  fp64        FP64 forces from the FP64 state, FP64 x, v, a (nbgb_system with
              NBGB_FLAG_FP64).
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib, ics
from .api import (FLAG_COMPENSATED, FLAG_FP64, FLAG_SYNC, DirectForceCalculator, Integrator,
                  ScopedParticleData, System, check)

__all__ = ["VARIANTS", "force_errors", "energy_drift"]

VARIANTS = ("fp32", "fp32c_fp64", "fp64")


def _flags(variant: str) -> int:
    return {"fp32": FLAG_SYNC, "fp32c_fp64": FLAG_SYNC | FLAG_COMPENSATED,
            "fp64": FLAG_SYNC | FLAG_FP64}[variant]


def _calc(variant: str, eps: float) -> DirectForceCalculator:
    c = DirectForceCalculator()
    c.setSofteningParameter(eps)
    c.set_flags(_flags(variant))
    return c


def _fp64_reference(s: dict, targets: np.ndarray, eps: float) -> np.ndarray:
    import torch
    n = len(s["x"])
    src = torch.from_numpy(np.stack([s["x"], s["y"], s["z"], s["m"]], axis=1).astype(np.float32)
                           .copy()).cuda()
    tg = torch.from_numpy(targets.astype(np.int64)).cuda()
    out = [torch.empty(len(targets), dtype=torch.float64, device="cuda") for _ in range(3)]
    check(_lib.lib().nbgb_direct_f64(C.c_void_p(src.data_ptr()), n, C.c_void_p(tg.data_ptr()),
                                     len(targets), 1.0, eps, *(C.c_void_p(o.data_ptr()) for o in out),
                                     None))
    torch.cuda.synchronize()
    return np.stack([o.cpu().numpy() for o in out], axis=1)


def _vec_rel(a: np.ndarray, ref: np.ndarray) -> np.ndarray:
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)


def force_errors(n: int, eps: float, seed: int = 1, samples: int = 4096) -> dict:
    s = ics.plummer(n, seed=seed)
    rng = np.random.Generator(np.random.PCG64(seed + 1000))
    targets = np.sort(rng.choice(n, size=min(samples, n), replace=False))
    ref = _fp64_reference(s, targets, eps)
    out = {}
    for variant in ("fp32", "fp32c_fp64"):
        calc = _calc(variant, eps)
        with ScopedParticleData(n, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                    "mass": s["m"]}) as p:
            calc.computeForces(p.device)
            p.download()
            a = np.stack([p.host[k][targets].astype(np.float64)
                          for k in ("acc_x", "acc_y", "acc_z")], axis=1)
        calc.close()
        e = _vec_rel(a, ref)
        out[variant] = {"median": float(np.median(e)), "p99": float(np.quantile(e, 0.99)),
                        "max": float(e.max())}
    # the full-FP64 variant computes this reference sum itself
    out["fp64"] = {"median": 0.0, "p99": 0.0, "max": 0.0, "note": "is the FP64 reference"}
    return {"n": n, "eps": eps, "samples": int(len(targets)), "variants": out}


def _energy_of(state: dict, eps: float) -> float:
    calc = DirectForceCalculator()
    calc.setSofteningParameter(eps)
    sysm = System(calc, state)
    ke, pe, _ = sysm.energy()
    sysm.close()
    calc.close()
    return ke + pe


def energy_drift(n: int, eps: float, dt: float, steps: int, seed: int = 1,
                 variants=VARIANTS) -> dict:
    import torch
    s = ics.plummer(n, seed=seed)
    out = {}
    e0 = None
    for variant in variants:
        if variant == "fp32":
            calc = _calc(variant, eps)
            integ = Integrator()
            arr = {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"], "vel_x": s["vx"],
                   "vel_y": s["vy"], "vel_z": s["vz"], "mass": s["m"]}
            with ScopedParticleData(n, arr) as p:
                if e0 is None:
                    e0 = _energy_of(s, eps)
                calc.computeForces(p.device)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for _ in range(steps):
                    integ.integrate(p.device, calc, dt)
                torch.cuda.synchronize()
                el = time.perf_counter() - t0
                p.download()
                fin = {"x": p.host["pos_x"], "y": p.host["pos_y"], "z": p.host["pos_z"],
                       "vx": p.host["vel_x"], "vy": p.host["vel_y"], "vz": p.host["vel_z"],
                       "m": s["m"]}
                fin = {k: v.copy() for k, v in fin.items()}
            calc.close()
            e1 = _energy_of(fin, eps)
        else:
            calc = _calc(variant, eps)
            sysm = System(calc, s)
            ke, pe, _ = sysm.energy()
            if e0 is None:
                e0 = ke + pe
            t0 = time.perf_counter()
            sysm.step(dt, steps)
            el = time.perf_counter() - t0
            ke, pe, _ = sysm.energy()
            e1 = ke + pe
            sysm.close()
            calc.close()
        out[variant] = {"dE_over_E": float(abs(e1 - e0) / abs(e0)), "E0": e0, "E1": e1,
                        "ms_per_step": 1e3 * el / steps}
    return {"n": n, "eps": eps, "dt": dt, "steps": steps, "variants": out}
