#!/usr/bin/env python3
"""Ensemble-serving benchmark on one GB300 (one JSON line on stdout).

Workload (synthetic, seeded): a stream of independent Plummer clusters
(a = 1, M = 1, G = 1) with N log-uniform in [256, 65536], step counts uniform
in [100, 2000], eps = 0.01, dt = 1e-3; direct sum for N <= 8192, Barnes-Hut
theta = 0.5 otherwise; FP32 forces, FP64 x/v state; 64 GiB admission budget.

  value   batched particle-steps/s: `--steps` ticks of the continuous-batching
          engine at saturation (resident cap `--resident`, backlog queued),
          timed with CUDA events on the engine stream;
  plain   the same requests run one at a time through the plain device path
          (nbgb_system per request), particle-steps/s;
  serve   Poisson arrivals at 80 % of the measured capacity: p50/p99 request
          latency (arrival -> result on the host) and e2e particle-steps/s
          through the public API (host arrays in, host results out).

`--impl reference` times the reference's CPU path for the same workload (the
CPU restatement in oracle/, all host threads).  Multi-GPU: one replica per
rank on its own shard of the request stream (weak scaling), max time over
ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "nbody-gpu-sim_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "batched vs plain particle-steps/s on 1 GB300 at stated force err; p99 latency"
UNIT = "particle-steps/s"
WORKLOAD = ("ensemble serving: Plummer clusters (a=1, M=1), N log-uniform [256, 65536], "
            "steps U[100, 2000], eps=0.01, dt=1e-3, direct N<=8192 else Barnes-Hut theta=0.5, "
            "FP32 forces + FP64 state, 64 GiB admission budget")
DT = 1e-3
EPS = 0.01
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=150, help="timed engine ticks")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="nbgb", choices=["nbgb", "reference"])
    ap.add_argument("--resident", type=int, default=96, help="resident systems at saturation")
    ap.add_argument("--plain-requests", type=int, default=48)
    ap.add_argument("--plain-steps", type=int, default=20)
    ap.add_argument("--e2e-ticks", type=int, default=600,
                    help="ticks of the saturated end-to-end run")
    ap.add_argument("--serve-requests", type=int, default=4096,
                    help="requests of the Poisson serving run (the workload's stream)")
    ap.add_argument("--serve-max-s", type=float, default=900.0)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-budget-s", type=float, default=120.0,
                    help="--impl reference: CPU seconds spread over warmup + steps")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--reference-walk", action="store_true",
                    help="serve Barnes-Hut systems with the reference's per-target walk")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--case", choices=["direct", "bh", "bh8", "bhg", "bhg8", "hash", "integrate",
                                       "precision"], default=None,
                    help="time one plain force evaluation of a single system instead "
                         "(small profiling cases), or run the precision study")
    ap.add_argument("--case-n", type=int, default=None,
                    help="bodies of a --case run (262144; 33554432 for integrate)")
    ap.add_argument("--stage-times", action="store_true",
                    help="with --case: device milliseconds per stage of the timed evaluations "
                         "(NBGB_FLAG_STAGE_TIMINGS)")
    ap.add_argument("--precision-steps", type=int, default=2000)
    ap.add_argument("--precision-fp64-steps", type=int, default=16,
                    help="steps of the three-variant run at the full N of --case precision")
    return ap.parse_args()


def precision_arm(args, local) -> dict:
    """Precision study on a Plummer sphere (a=1, M=1), eps=1e-3, dt=2^-10:
    force error of FP32 plain and FP32 compensated against the FP64 direct
    sum at N=262144 (4096 seeded targets); energy drift over 2000 steps of
    both FP32 variants at N=262144 and of all three variants (with full
    FP64) at N=16384, where FP64 arithmetic fits the time budget; and all
    three variants at N=262144 over a reduced step count
    (--precision-fp64-steps, 16 by default: one FP64 step takes ~5 s there)."""
    import torch

    import nbgb.precision as prec
    torch.cuda.set_device(local)
    eps, dt = 1e-3, 2.0 ** -10
    steps = args.precision_steps
    n = args.case_n or 262144
    out = {"case": "precision", "force_error": prec.force_errors(n, eps),
           "energy_full_n": prec.energy_drift(n, eps, dt, steps,
                                              variants=("fp32", "fp32c_fp64")),
           "energy_small_n": prec.energy_drift(16384, eps, dt, steps)}
    if args.precision_fp64_steps > 0:
        out["energy_full_n_all_variants"] = prec.energy_drift(n, eps, dt,
                                                              args.precision_fp64_steps)
    return out


def case_arm(args, local):
    """One system through nbgb_compute_forces: direct / Barnes-Hut (theta 0.5;
    1 or 8 bodies per leaf, with the reference-style walk or the group walk)
    on a Plummer sphere, or the
    spatial hash on the uniform cube at the serving density; prints ms per
    evaluation."""
    import torch

    import nbgb
    torch.cuda.set_device(local)
    n = args.case_n or 262144
    if args.case == "hash":
        side = 160.0 * (n / 4_194_304) ** (1.0 / 3.0)
        s = nbgb.ics.uniform_cube(n, seed=3, side=side)
        calc = nbgb.SpatialHashCalculator(2.0, 2.0)
    elif args.case == "direct":
        s = nbgb.ics.plummer(n, seed=1)
        calc = nbgb.DirectForceCalculator()
    else:
        s = nbgb.ics.two_plummer(n, seed=2)
        calc = nbgb.BarnesHutCalculator(0.5, leaf_capacity=8 if args.case in ("bh8", "bhg8") else 1,
                                        group_walk=args.case in ("bhg", "bhg8"))
    calc.setSofteningParameter(EPS)
    if args.stage_times:
        calc.set_flags(calc.params.flags | nbgb.FLAG_STAGE_TIMINGS)
    st = torch.cuda.current_stream()
    calc.set_stream(st.cuda_stream)
    with nbgb.ScopedParticleData(n, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                     "mass": s["m"]}) as p:
        for _ in range(max(args.warmup, 1)):
            calc.computeForces(p.device)
        torch.cuda.synchronize()
        if args.stage_times:
            calc.stage_times(reset=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.steps):
            calc.computeForces(p.device)
        e1.record(st)
        torch.cuda.synchronize()
        stages = calc.stage_times() if args.stage_times else None
    calc.close()
    out = {"case": args.case, "n": n, "ms_per_eval": e0.elapsed_time(e1) / args.steps}
    if stages:
        out["stage_ms_per_eval"] = {k: round(v[0] / max(v[1], 1), 4) for k, v in stages.items()}
    return out


def per_config_timings(nbgb) -> dict:
    """The single-system workloads of the other configurations, timed in the
    same run (CUDA events over 10 force evaluations after 2 warm-ups, inputs
    resident; the median of three such batches): Barnes-Hut on two Plummer
    spheres N = 1,048,576 (theta 0.5, eps 0.01) with the reference-style
    walk and with the group walk, one body per leaf and 8-body buckets (the
    workload's leaf <= 8); the spatial hash on the uniform cube N = 4,194,304
    (cell = cutoff = 2)."""
    import torch

    def timed(calc, s, reps=10):
        calc.setSofteningParameter(EPS)
        st = torch.cuda.current_stream()
        calc.set_stream(st.cuda_stream)
        n = len(s["x"])
        with nbgb.ScopedParticleData(n, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                         "mass": s["m"]}) as p:
            for _ in range(2):
                calc.computeForces(p.device)
            torch.cuda.synchronize()
            batches = []
            for _ in range(3):
                e0, e1 = (torch.cuda.Event(enable_timing=True),
                          torch.cuda.Event(enable_timing=True))
                e0.record(st)
                for _ in range(reps):
                    calc.computeForces(p.device)
                e1.record(st)
                torch.cuda.synchronize()
                batches.append(e0.elapsed_time(e1) / reps)
        calc.close()
        return sorted(batches)[1]

    out = {}
    s = nbgb.ics.two_plummer(1 << 20, seed=2)
    bh = {}
    for name, leaf, group in (("reference_walk_leaf1", 1, False), ("reference_walk_leaf8", 8, False),
                              ("group_walk_leaf1", 1, True), ("group_walk_leaf8", 8, True)):
        bh[name] = timed(nbgb.BarnesHutCalculator(0.5, leaf_capacity=leaf, group_walk=group), s)
    out["barnes_hut_two_plummer_1048576_ms_per_eval"] = bh
    del s
    s = nbgb.ics.uniform_cube(4_194_304, seed=3, side=160.0)
    out["spatial_hash_uniform_4194304_ms_per_eval"] = timed(nbgb.SpatialHashCalculator(2.0, 2.0), s)
    return out


def integrate_arm(args, local):
    """Achieved HBM bandwidth of the reference-semantics integrator kernels
    (updatePositions, updateVelocities, storeOldAccelerations of
    src/cuda/integrator.cu:12-49) through the public Integrator, on N bodies
    whose arrays (52 B/body, 1.7 GB at the default N) exceed L2, so nothing is
    flushed between launches.  Algorithmic bytes per body: positions 36 read
    (pos, vel, acc) + 12 written; velocities 36 read (vel, acc_old, acc) + 12
    written; store-old 12 read + 12 written.  Peak: the measured copy
    bandwidth (read + write bytes) of MEASURED_PEAKS.json."""
    import torch

    import nbgb
    torch.cuda.set_device(local)
    n = args.case_n or (1 << 25)
    rng = np.random.Generator(np.random.PCG64(9))
    arrays = {k: rng.standard_normal(n, dtype=np.float32)
              for k in ("pos_x", "pos_y", "pos_z", "vel_x", "vel_y", "vel_z",
                        "acc_x", "acc_y", "acc_z")}
    arrays["mass"] = np.full(n, 1.0 / n, np.float32)
    peak = measured_peaks().get("hbm_gbs")
    integ = nbgb.Integrator()
    st = torch.cuda.current_stream()  # the legacy stream the Integrator launches on
    out = {"case": "integrate", "n": n, "peak_gbs": peak,
           "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy, read + write)"}
    with nbgb.ScopedParticleData(n, arrays) as p:
        kernels = (("vv_positions_kernel", lambda: integ.updatePositions(p.device, DT), 48),
                   ("vv_velocities_kernel", lambda: integ.updateVelocities(p.device, DT), 48),
                   ("store_old_kernel", lambda: integ.storeOldAccelerations(p.device), 24))
        for name, fn, bpb in kernels:
            for _ in range(max(args.warmup, 3)):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(args.steps):
                fn()
            e1.record(st)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            gbs = bpb * n / (ms / 1e3) / 1e9
            out[name] = {"ms": ms, "bytes_per_body": bpb, "achieved_gbs": gbs,
                         "frac": gbs / peak if peak else None}
    return out


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class Clocks:
    """nvidia-smi samples every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int) -> None:
        self.idx = gpu_index
        self.rows: list[list[str]] = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> dict:
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def make_state(nbgb, req):
    return nbgb.ics.plummer(req["n"], seed=req["seed"])


def request_work(reqs) -> float:
    return float(sum(r["n"] * r["steps"] for r in reqs))


# ----------------------------------------------------------------- GPU arm --
def gpu_arm(args, rank, world, local):
    import ctypes as C

    import torch

    import nbgb
    from nbgb.serving import Ensemble, serve

    torch.cuda.set_device(local)
    dev_index = torch.cuda.current_device()
    lib = nbgb.lib()
    ffma, ffma2, mufu = C.c_double(), C.c_double(), C.c_double()
    nbgb.check(lib.nbgb_measure_fp32_peak(C.byref(ffma), C.byref(ffma2), C.byref(mufu)))

    stream_seed = shard_seed(rank)
    stream = nbgb.ics.ensemble_requests(4096, seed=stream_seed)
    S = args.resident
    # --- batched, saturation --------------------------------------------------
    backlog = stream[: S + 256]
    states = {r["id"]: make_state(nbgb, r) for r in backlog}
    walk = 0 if args.reference_walk else 1
    ens = Ensemble(hbm_budget_bytes=64 << 30, max_resident=S, softening=EPS, theta=0.5,
                   group_walk=walk)
    for r in backlog:
        ens.submit(states[r["id"]], r["steps"], DT)
    prime = 0
    while True:  # admission + autotuning outside the measurement
        ens.tick()
        prime += 1
        if (ens.stats()["tuning"] == 0 and prime >= 3) or prime >= 60:
            break
    for _ in range(args.warmup):
        ens.tick()
    est = torch.cuda.ExternalStream(ens.stream())
    s0 = ens.stats()
    resident_bytes = s0["bytes_reserved"]
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # clocks sampled every 100 ms over the timed ticks and the end-to-end run
    # right after them (both under load)
    clk = Clocks(dev_index).__enter__()
    torch.cuda.nvtx.range_push("bench_timed")  # profilers can filter on this range
    e0.record(est)
    t_host = time.perf_counter()
    for _ in range(args.steps):
        ens.tick()
    e1.record(est)
    torch.cuda.synchronize()
    host_s = time.perf_counter() - t_host
    torch.cuda.nvtx.range_pop()
    elapsed_s = e0.elapsed_time(e1) / 1e3
    s1 = ens.stats()
    ps = s1["particle_steps"] - s0["particle_steps"]
    dint = s1["direct_kernel_interactions"] - s0["direct_kernel_interactions"]
    dms = s1["direct_kernel_ms"] - s0["direct_kernel_ms"]
    bh_int = s1["bh_interactions"] - s0["bh_interactions"]
    walk_ms = s1["bh_walk_ms"] - s0["bh_walk_ms"]
    bh_bodies = s1["bh_bodies"]
    launches = s1["kernel_launches"] - s0["kernel_launches"]
    tuned = s1["direct_config"]
    ens.close()
    # --- end to end at saturation: host arrays in, results read back ----------
    e2e_rep = e2e_arm(nbgb, Ensemble, backlog, states, S, tuned, args.e2e_ticks, world, walk)
    clk.__exit__(None, None, None)
    del states

    # --- reduction over ranks ---------------------------------------------------
    t_max, ps_tot = reduce_over_ranks(elapsed_s, ps, world)
    value = ps_tot / t_max

    out = {}
    if rank == 0:
        # --- plain: one request at a time --------------------------------------
        plain = None
        if not args.no_plain:
            plain = plain_arm(nbgb, stream[: args.plain_requests], args.plain_steps)
        # --- serving: Poisson arrivals at 80 % load, latency, e2e ---------------
        serve_rep = None
        if not args.no_serve:
            sreqs = nbgb.ics.ensemble_requests(args.serve_requests, seed=stream_seed + 7)
            work = request_work(sreqs) / len(sreqs)  # particle-steps per request
            rate = 0.8 * value / work  # requests per second at 80 % of capacity
            for r in sreqs:
                r["arrival"] = r["arrival"] / rate  # unit-rate stream -> target rate
            cache = {}

            def mk(req):
                st = cache.pop(req["id"], None)
                return st if st is not None else make_state(nbgb, req)

            for r in sreqs[:64]:
                cache[r["id"]] = make_state(nbgb, r)
            ens2 = Ensemble(hbm_budget_bytes=64 << 30, softening=EPS, theta=0.5)
            rep = serve(ens2, sreqs, mk, dt=DT, time_scale=1.0, max_wall_s=args.serve_max_s)
            ens2.close()
            h2d = sum(7 * 4 * r["n"] for r in sreqs)
            d2h = sum((6 * 8 + 4 * 4) * r["n"] for r in sreqs)
            serve_rep = dict(rate_req_s=rate, completed=rep.completed, offered=len(sreqs),
                             wall_s=rep.wall_s, particle_steps=rep.particle_steps,
                             particle_steps_per_s=rep.particle_steps / rep.wall_s,
                             ticks=rep.ticks, p50_s=rep.percentile(50), p99_s=rep.percentile(99),
                             h2d=h2d, d2h=d2h)
        # --- CPU baseline (reference CPU path, restated) -------------------------
        cpu = cpu_baseline(nbgb, stream, args.cpu_seconds)
        cpu["direct_n1024_100_steps"] = c1_cpu_baseline(nbgb)
        per_config = per_config_timings(nbgb)
        force_err = measured_force_error(nbgb)

        ffma_peak = ffma.value
        d_achieved = 20.0 * dint / (dms / 1e3) / 1e12 if dms > 0 else None
        w_achieved = 20.0 * bh_int / (walk_ms / 1e3) / 1e12 if walk_ms > 0 else None
        walk_share = (walk_ms / 1e3) / elapsed_s if elapsed_s > 0 else None
        direct_share = (dms / 1e3) / elapsed_s if elapsed_s > 0 else None
        # DRAM bytes of the walk: ncu capture (dram__bytes_read.sum +
        # dram__bytes_write.sum) of the group-walk launch of the first timed
        # tick of this workload, 341.7 MB + 36.1 MB for 1,179,805 bodies
        # walked, scaled by the bodies walked here
        walk_traffic = 377.85e6 / 1179805 * bh_bodies if bh_bodies else None
        clocks = clk.summary()
        clocks["window"] = "timed ticks and the saturated end-to-end run"
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Plummer clusters; no dataset)",
            "config": {
                "workload": WORKLOAD, "resident_systems": S, "backlog_requests": len(backlog),
                "tick": "one Velocity-Verlet step of every resident system",
                "l2": f"not flushed; resident state + trees {resident_bytes / 2**20:.0f} MiB > "
                      f"L2 {L2_BYTES / 2**20:.0f} MiB",
                "direct_kernel_config": tuned, "theta": 0.5, "softening": EPS, "dt": DT,
                "force_error": "direct: compensated FP32, median rel err ~1e-7 vs FP64; "
                               "Barnes-Hut theta=0.5 group walk (each accepted cell passes "
                               "the reference's per-target test for every body of its "
                               "group): median rel err <= 1e-3 vs FP64, below the reference "
                               "walk's (tests/test_bh_gpu.py, tests/test_direct_gpu.py); "
                               "measured on served systems: force_error_measured",
                "bh_walk": ("group walk (NBGB_FLAG_GROUP_WALK); the plain runs use the same"
                            if walk else "the reference's per-target walk (--reference-walk) "
                            "in the timed and end-to-end runs"),
                "parallelism": f"replicas x{world} (request-stream shards)",
            },
            "force_error_measured": force_err,
            "batched_particle_steps_per_s": value,
            "plain_particle_steps_per_s": plain["value"] if plain else None,
            "batched_vs_plain": (value / world / plain["value"]) if plain else None,
            "plain": plain,
            "interactions_per_s": (dint + bh_int) / t_max,
            "direct_interactions_per_s": dint / t_max,
            "bh_interactions_per_s": bh_int / t_max,
            "host_s": host_s,
            "latency_p50_s": serve_rep["p50_s"] if serve_rep else None,
            "latency_p99_s": serve_rep["p99_s"] if serve_rep else None,
            "serve": serve_rep,
            "e2e": {"value": e2e_rep["value"], "unit": UNIT,
                    "h2d_bytes_per_step": e2e_rep["h2d_bytes_per_step"],
                    "d2h_bytes_per_step": e2e_rep["d2h_bytes_per_step"],
                    "ticks": e2e_rep["ticks"], "wall_s": e2e_rep["wall_s"],
                    "results_read": e2e_rep["results_read"], "admitted": e2e_rep["admitted"],
                    "note": "saturated serving through the public API (host clock): host "
                            "arrays submitted and copied in at admission, every finished "
                            "request's state polled back to the host; latency is measured "
                            "separately under Poisson arrivals at 80% load (serve)"},
            "roofline": {
                "kernel": "bh_group_walk_kernel (batched Barnes-Hut group walk, all resident "
                          "BH systems)",
                "bound": "fp32", "achieved": w_achieved, "peak": ffma_peak, "unit": "TFLOP/s",
                "frac": (w_achieved / ffma_peak) if w_achieved else None,
                "traffic": walk_traffic,
                "traffic_source": "ncu dram__bytes_read+write of the group-walk launch of the "
                                  "first timed tick of this workload (377.9 MB for 1,179,805 "
                                  "bodies walked), scaled by the bodies walked",
                "algorithmic_bytes": 64 * 1.5 * bh_bodies + 28 * bh_bodies if bh_bodies else None,
                "peak_source": "measured in-process: FFMA chains on every SM "
                               "(nbgb_measure_fp32_peak); MEASURED_PEAKS.json has no FP32 figure",
                "flops_per_interaction": 20, "share_of_tick": walk_share,
                "walk_ms_per_tick": walk_ms / args.steps,
                "note": "list evaluation in packed FP32x2, two bodies per lane in groups "
                        "of up to 64, and a latency-bound traversal: FMA pipe 64 %, issue "
                        "65 %, warps active 35 % at 80 registers (ncu, N=1M two-Plummer); "
                        "interactions counted per body (list length minus the body "
                        "itself)",
                "hbm_peak_gbs_measured": measured_peaks().get("hbm_gbs"),
            },
            "direct_kernel": {"kernel": "ens_direct_kernel (direct-sum work queue)",
                              "achieved_tflops": d_achieved, "share_of_tick": direct_share,
                              "note": "overlaps the Barnes-Hut chain on another stream"},
            "fp32_peaks": {"ffma_tflops": ffma.value, "ffma2_tflops": ffma2.value,
                           "mufu_gops": mufu.value,
                           "spec_tflops": spec_fp32_tflops(clocks.get("sm_max_mhz")),
                           "spec_note": "SMs x 128 FP32 lanes x 2 flops x the maximum SM "
                                        "clock (nvidia-smi)"},
            "cpu_baseline": cpu,
            "per_config": per_config,
            "clocks": clocks,
            "gpu_launches": launches,
        }
    return out


def spec_fp32_tflops(sm_max_mhz) -> float | None:
    """Nominal FP32 FMA rate: SMs x 128 lanes x 2 flops x clock."""
    if not sm_max_mhz:
        return None
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    return sms * 128 * 2 * float(sm_max_mhz) * 1e6 / 1e12


def measured_force_error(nbgb) -> dict:
    """Force error of the ensemble's accelerations as served: one direct
    (N = 6000) and one Barnes-Hut (N = 30000) system of the serving workload
    run 3 steps in one engine; their final accelerations are compared with
    the FP64 direct sum at the final FP32 positions (nbgb_direct_f64) on
    2048 seeded targets each (vector relative error)."""
    import ctypes as C

    import torch

    from nbgb.serving import Ensemble
    ens = Ensemble(hbm_budget_bytes=4 << 30, softening=EPS, theta=0.5)
    sys_ = {ens.submit(nbgb.ics.plummer(6000, seed=901), 3, DT): "direct",
            ens.submit(nbgb.ics.plummer(30000, seed=902), 3, DT): "barnes_hut"}
    for _ in range(20):
        if ens.tick() == (0, 0):
            break
    ens.synchronize()
    out = {}
    while (r := ens.poll(want_state=True, want_acc=True)) is not None:
        s = r[1]
        n = len(s["m"])
        xyzm = np.stack([s["x"].astype(np.float32), s["y"].astype(np.float32),
                         s["z"].astype(np.float32), s["m"]], 1)
        src = torch.from_numpy(np.ascontiguousarray(xyzm)).cuda()
        tg = np.sort(np.random.default_rng(n).choice(n, 2048, replace=False)).astype(np.int64)
        tgd = torch.from_numpy(tg).cuda()
        acc = [torch.empty(len(tg), dtype=torch.float64, device="cuda") for _ in range(3)]
        nbgb.check(nbgb.lib().nbgb_direct_f64(C.c_void_p(src.data_ptr()), n,
                                               C.c_void_p(tgd.data_ptr()), len(tg), 1.0, EPS,
                                               *(C.c_void_p(a.data_ptr()) for a in acc), None))
        torch.cuda.synchronize()
        ref = np.stack([a.cpu().numpy() for a in acc], 1)
        got = np.stack([s["ax"][tg], s["ay"][tg], s["az"][tg]], 1).astype(np.float64)
        e = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
        out[sys_[r[0]["request_id"]]] = {"n": n, "median": float(np.median(e)),
                                         "p99": float(np.quantile(e, 0.99))}
    ens.close()
    return out


def e2e_arm(nbgb, Ensemble, reqs, states, S, direct_config, ticks, world, walk=1) -> dict:
    """The saturated serving loop through the public API: requests are
    submitted as host arrays (copied to the device at admission), the engine is
    ticked, and every finished request's state is polled back to the host
    (FP64 positions and velocities, FP32 accelerations and masses).  The queue
    is kept S + 32 deep by resubmitting the prepared requests in turn, so the
    resident set stays full.  Timed on the host clock over `ticks` ticks, the
    submits, polls and copies included, synchronised at both ends."""
    import itertools
    ens = Ensemble(hbm_budget_bytes=64 << 30, max_resident=S, softening=EPS, theta=0.5,
                   direct_config=direct_config, group_walk=walk)
    feed = itertools.cycle(reqs)
    outstanding, h2d, d2h, results = 0, 0, 0, 0

    def top_up():
        nonlocal outstanding, h2d
        while outstanding < S + 32:
            r = next(feed)
            ens.submit(states[r["id"]], r["steps"], DT)
            h2d += 7 * 4 * r["n"]  # x y z vx vy vz m, FP32
            outstanding += 1

    def drain():
        nonlocal outstanding, d2h, results
        while (got := ens.poll(want_state=True)) is not None:
            res, _ = got
            d2h += (6 * 8 + 4 * 4) * res["count"]
            outstanding -= 1
            results += 1

    top_up()
    for _ in range(8):  # admission, first build, graph capture
        ens.tick()
        drain()
        top_up()
    ens.synchronize()
    s0 = ens.stats()
    h2d = d2h = results = 0
    t0 = time.perf_counter()
    for _ in range(ticks):
        top_up()
        ens.tick()
        drain()
    ens.synchronize()
    drain()
    wall = time.perf_counter() - t0
    s1 = ens.stats()
    ens.close()
    ps = s1["particle_steps"] - s0["particle_steps"]
    t_max, ps_tot = reduce_over_ranks(wall, ps, world)
    return {"value": ps_tot / t_max, "ticks": ticks, "wall_s": t_max, "results_read": results,
            "admitted": s1["admitted"] - s0["admitted"],
            "h2d_bytes_per_step": h2d / ticks, "d2h_bytes_per_step": d2h / ticks}


def plain_arm(nbgb, reqs, steps) -> dict:
    """Each request alone through the plain device path, in sequence: the
    device-resident FP64 system with asynchronous calculators (no per-step
    host synchronisation; one at the end)."""
    tot_ps, tot_s = 0.0, 0.0
    per = []
    for r in reqs:
        s = make_state(nbgb, r)
        if r["n"] <= 8192:
            calc = nbgb.DirectForceCalculator()
        else:  # the serving engine's walk, so both runs have the same accuracy
            calc = nbgb.BarnesHutCalculator(0.5, group_walk=True)
        calc.setSofteningParameter(EPS)
        # asynchronous: no per-step read-back
        calc.set_flags(calc.params.flags & ~nbgb.FLAG_SYNC)
        sysm = nbgb.System(calc, s)
        sysm.step(DT, 2)  # warm
        calc.synchronize()
        t0 = time.perf_counter()
        sysm.step(DT, steps)
        calc.synchronize()
        dt = time.perf_counter() - t0
        sysm.close()
        calc.close()
        tot_ps += r["n"] * steps
        tot_s += dt
        per.append((r["n"], dt / steps))
    return {"value": tot_ps / tot_s, "requests": len(reqs), "steps_each": steps,
            "ms_per_step_by_n": [[n, 1e3 * t] for n, t in per[:12]]}


def cpu_step(orc, nbgb, r) -> tuple[float, float]:
    """One Velocity-Verlet step of request r on the host through the
    reference's CPU path as restated in oracle/ (src/cuda/integrator.cu:12-37
    update formulae around the forces: pair-function direct sum in reference
    order for N <= 8192; the reference insertion octree + per-target walk for
    the Barnes-Hut systems).  a(t) comes from a force evaluation before the
    timer (direct) or is zero (Barnes-Hut: the update's cost does not depend
    on its values).  Returns (particle-steps, seconds)."""
    s = make_state(nbgb, r)
    x, y, z, m = s["x"].copy(), s["y"].copy(), s["z"].copy(), s["m"]
    vx, vy, vz = s["vx"].copy(), s["vy"].copy(), s["vz"].copy()
    n = r["n"]
    if n <= 8192:
        ax, ay, az = orc.direct_f32(x, y, z, m, 1.0, EPS)  # a(t) of a running system

        def forces():
            return orc.direct_f32(x, y, z, m, 1.0, EPS)
    else:
        ax, ay, az = (np.zeros(n, np.float32) for _ in range(3))

        def forces():
            bmin, bmax = orc.bbox(x, y, z)
            _, si = orc.stable_sort(*orc.morton_keys(x, y, z, bmin, bmax))
            nodes, _, _ = orc.build_octree(x, y, z, m, si, bmin, bmax)
            return orc.bh_forces(nodes, x, y, z, m, 0.5, 1.0, EPS)[:3]
    t0 = time.perf_counter()
    ox, oy, oz = ax.copy(), ay.copy(), az.copy()
    orc.update_positions(x, y, z, vx, vy, vz, ax, ay, az, DT)
    ax, ay, az = (np.ascontiguousarray(a, np.float32) for a in forces())
    orc.update_velocities(vx, vy, vz, ox, oy, oz, ax, ay, az, DT)
    return float(n), time.perf_counter() - t0


def c1_cpu_baseline(nbgb) -> dict:
    """The plain direct workload on the host: N = 1024 Plummer sphere, 100
    Velocity-Verlet steps, eps = 0.01, dt = 1e-3, the reference's pair
    function in its order (src/cuda/force_direct.cu:109-117) and update
    formulae (src/cuda/integrator.cu:12-37), restated in oracle/; timed on one
    core and on all host cores."""
    from oracle.oracle import Oracle
    orc = Oracle()
    s = nbgb.ics.plummer(1024, seed=1)
    all_threads = orc.num_threads()
    out = {"workload": "Plummer N=1024, 100 Velocity-Verlet steps, eps=0.01, dt=1e-3",
           "host_cores": os.cpu_count()}
    for label, threads in (("one_core", 1), ("all_cores", all_threads)):
        orc.set_num_threads(threads)
        x, y, z, m = (s[k].copy() for k in ("x", "y", "z", "m"))
        vx, vy, vz = (s[k].copy() for k in ("vx", "vy", "vz"))
        ax, ay, az = orc.direct_f32(x, y, z, m, 1.0, EPS)
        t0 = time.perf_counter()
        for _ in range(100):
            ox, oy, oz = ax, ay, az
            orc.update_positions(x, y, z, vx, vy, vz, ax, ay, az, DT)
            ax, ay, az = orc.direct_f32(x, y, z, m, 1.0, EPS)
            orc.update_velocities(vx, vy, vz, ox, oy, oz, ax, ay, az, DT)
        dt = time.perf_counter() - t0
        out[label] = {"threads": threads, "seconds": dt, "ms_per_step": 10.0 * dt,
                      "particle_steps_per_s": 1024 * 100 / dt,
                      "interactions_per_s": 1024 * 1023 * 100 / dt}
    orc.set_num_threads(all_threads)
    return out


def cpu_baseline(nbgb, stream, seconds) -> dict:
    """The reference's CPU path on a bounded sample of the request stream,
    one step per sampled system (cpu_step)."""
    from oracle.oracle import Oracle
    orc = Oracle()
    ps, t = 0.0, 0.0
    count = 0
    for r in stream:
        if t > seconds:
            break
        p, dt = cpu_step(orc, nbgb, r)
        ps += p
        t += dt
        count += 1
    return {"value": ps / t if t > 0 else None, "unit": UNIT, "cores": orc.num_threads(),
            "kind": "port",
            "sample": f"{count} systems of the same request stream, one Velocity-Verlet step "
                      f"each on the host (direct: reference pair function order; N>8192: "
                      f"reference insertion octree + walk), {t:.1f} s of CPU time"}


# ------------------------------------------------------------ multi-rank --
def shard_seed(rank: int) -> int:
    """Seed of rank's own shard of the request stream (weak scaling: every
    rank serves an independent stream of the same distribution)."""
    return 5 + 1000 * rank


def reduce_over_ranks(elapsed_s: float, particle_steps: float, world: int) -> tuple[float, float]:
    """(max elapsed over ranks, particle-steps summed over ranks); the only
    collectives of the benchmark (no data-path exchange)."""
    if world <= 1:
        return elapsed_s, float(particle_steps)
    import torch
    import torch.distributed as dist
    tt = torch.tensor([elapsed_s], dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    pt = torch.tensor([float(particle_steps)], dtype=torch.float64)
    dist.all_reduce(pt, op=dist.ReduceOp.SUM)
    return float(tt.item()), float(pt.item())


# ----------------------------------------------------------- reference arm --
def reference_arm(args, rank, world):
    """The reference's CPU path (cpu_step) on the host cores, rank 0 only:
    each step a bounded sample of the same request stream."""
    if rank != 0:
        return None
    import nbgb  # only for the request stream and the initial conditions
    stream = nbgb.ics.ensemble_requests(4096, seed=shard_seed(0))
    from oracle.oracle import Oracle
    orc = Oracle()
    per_step = min(20.0, max(0.5, args.ref_budget_s / max(args.steps + args.warmup, 1)))
    results = []
    idx = 0
    for k in range(args.warmup + args.steps):
        ps, t = 0.0, 0.0
        while t < per_step and idx < len(stream):
            p, dt = cpu_step(orc, nbgb, stream[idx])
            idx += 1
            ps += p
            t += dt
        if k >= args.warmup:
            results.append((ps, t))
    tot_ps = sum(p for p, _ in results)
    tot_t = sum(t for _, t in results)
    value = tot_ps / tot_t if tot_t > 0 else 0.0
    sample = (f"per step: consecutive systems of the request stream, one Velocity-Verlet "
              f"step each, ~{per_step:.1f} s of CPU work (direct: reference pair function "
              f"order; N>8192: reference insertion octree + walk)")
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot_t / max(len(results), 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Plummer clusters; no dataset)",
        "config": {"workload": WORKLOAD, "path": "reference host CPU path (restated)",
                   "bh_walk": "the reference's per-target walk on its insertion octree"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": orc.num_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main() -> int:
    args = parse()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.case == "precision":
        out = precision_arm(args, local) if rank == 0 else None
    elif args.case == "integrate":
        out = integrate_arm(args, local) if rank == 0 else None
    elif args.case:
        out = case_arm(args, local) if rank == 0 else None
    elif args.impl == "reference":
        out = reference_arm(args, rank, world)
    else:
        out = gpu_arm(args, rank, world, local)
    if rank == 0 and out:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
