"""Velocity Verlet through the C ABI vs the oracle (GPU).

Restates tests/test_integrator.cpp and checks trajectories of the Plummer
N = 1024 direct workload (100 steps, dt = 1e-3, eps = 0.01):
  * FP32 drop-in path vs the oracle's FP32 reference-formula integration:
    max |x - x_oracle| <= 1e-4;
  * FP64-state system path vs the FP64 oracle: max |x - x64| <= 2e-5 and
    |v - v64| <= 2e-4, energy drift |dE/E| <= 1e-5.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _one(v):
    return np.array([v], np.float32)


def test_single_step_position(nb):
    # tests/test_integrator.cpp:14-41
    with nb.ScopedParticleData(1, {"vel_x": _one(1.0), "mass": _one(1.0)}) as p:
        nb.Integrator().updatePositions(p.device, 0.1)
        p.download()
        assert abs(p.host["pos_x"][0] - 0.1) < 1e-5
        assert abs(p.host["pos_y"][0]) < 1e-5 and abs(p.host["pos_z"][0]) < 1e-5


def test_constant_acceleration_kinematics(nb):
    # :43-74
    arr = {"pos_x": _one(1.0), "pos_y": _one(-2.0), "pos_z": _one(0.5), "vel_x": _one(0.3),
           "vel_z": _one(-0.2), "acc_x": _one(2.0), "acc_y": _one(-1.0), "acc_z": _one(4.0),
           "mass": _one(1.0)}
    with nb.ScopedParticleData(1, arr) as p:
        dt = 0.01
        nb.Integrator().updatePositions(p.device, dt)
        p.download()
        h = p.host
        assert abs(h["pos_x"][0] - (1.0 + 0.3 * dt + 0.5 * 2.0 * dt * dt)) < 1e-6
        assert abs(h["pos_y"][0] - (-2.0 - 0.5 * dt * dt)) < 1e-6
        assert abs(h["pos_z"][0] - (0.5 - 0.2 * dt + 0.5 * 4.0 * dt * dt)) < 1e-6


def _fma32(a, b, c):
    # float32 fused multiply-add: the product of two floats is exact in
    # float64; the float64 sum then rounds to float32 (a double rounding that
    # differs from one rounding with probability ~2^-29 per element)
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def test_fp32_kernels_bitwise_ragged(nb):
    """storeOldAccelerations, updatePositions and updateVelocities on a
    ragged N against the reference formulas (integrator.cu:12-49) in float32
    with the device's rounding: x + fma(v, dt, a * (0.5 dt dt)) and
    v + (a_old + a) * (0.5 dt) with the final multiply-add fused.  acc_old is
    set on the device by storeOldAccelerations (the host copies carry pos,
    vel, acc and mass only, as the reference's).  Bit-exact."""
    n = (1 << 20) + 3
    rng = np.random.Generator(np.random.PCG64(17))
    keys = ("pos_x", "pos_y", "pos_z", "vel_x", "vel_y", "vel_z", "acc_x", "acc_y", "acc_z")
    arr = {k: rng.standard_normal(n, dtype=np.float32) for k in keys}
    arr["mass"] = rng.uniform(0.5, 1.5, n).astype(np.float32)
    new_acc = {c: rng.standard_normal(n, dtype=np.float32) for c in "xyz"}
    dt = np.float32(1e-2)
    integ = nb.Integrator()
    with nb.ScopedParticleData(n, arr) as p:
        integ.storeOldAccelerations(p.device)  # acc_old = the uploaded acc
        for c in "xyz":
            p.host["acc_" + c][:] = new_acc[c]
        p.upload()  # pos, vel, acc, mass; acc_old stays on the device
        integ.updatePositions(p.device, float(dt))
        integ.updateVelocities(p.device, float(dt))
        p.download()
        got = {k: p.host[k].copy() for k in keys}
    h2 = np.float32(np.float32(0.5) * dt) * dt
    hv = np.float32(0.5) * dt
    for c in "xyz":
        a, o = new_acc[c], arr["acc_" + c]
        want_x = arr["pos_" + c] + _fma32(arr["vel_" + c], np.full(n, dt), a * h2)
        np.testing.assert_array_equal(got["pos_" + c], want_x)
        want_v = _fma32(o + a, np.full(n, hv), arr["vel_" + c])
        np.testing.assert_array_equal(got["vel_" + c], want_v)
        np.testing.assert_array_equal(got["acc_" + c], a)


def test_kinetic_energy(nb):
    # :76-102
    arr = {"vel_x": np.array([1.0, 0.0], np.float32), "vel_y": np.array([0.0, 2.0], np.float32),
           "mass": np.array([1.0, 2.0], np.float32)}
    with nb.ScopedParticleData(2, arr) as p:
        assert abs(nb.Integrator().computeKineticEnergy(p.device) - 4.5) < 1e-4


def _orbit_state():
    r, G, m = 5.0, 1.0, 1.0
    v = np.sqrt(G * m / (4 * r))
    return {"pos_x": np.array([-r, r], np.float32), "vel_y": np.array([-v, v], np.float32),
            "mass": np.ones(2, np.float32)}


def test_two_body_orbit_energy_dropin(nb):
    # :107-168: r = 5, eps = 0.01, dt = 1e-3, 100 steps, |dE/E| < 1e-3
    calc = nb.DirectForceCalculator()
    calc.setGravitationalConstant(1.0)
    calc.setSofteningParameter(0.01)
    integ = nb.Integrator()
    with nb.ScopedParticleData(2, _orbit_state()) as p:
        calc.computeForces(p.device)
        e0 = integ.computeTotalEnergy(p.device, 1.0, 0.01)
        for _ in range(100):
            integ.integrate(p.device, calc, 0.001)
        e1 = integ.computeTotalEnergy(p.device, 1.0, 0.01)
        assert abs(e1 - e0) / abs(e0) < 1e-3
    calc.close()


def test_two_body_orbit_energy_system(nb):
    st = _orbit_state()
    s = {"x": st["pos_x"], "y": np.zeros(2, np.float32), "z": np.zeros(2, np.float32),
         "vx": np.zeros(2, np.float32), "vy": st["vel_y"], "vz": np.zeros(2, np.float32),
         "m": st["mass"]}
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(0.01)
    sysm = nb.System(calc, s)
    ke0, pe0, p0 = sysm.energy()
    sysm.step(0.001, 100)
    ke1, pe1, p1 = sysm.energy()
    e0, e1 = ke0 + pe0, ke1 + pe1
    assert abs(e1 - e0) / abs(e0) < 1e-5
    assert np.all(np.abs(p1 - p0) < 1e-9)
    sysm.close()
    calc.close()


def test_potential_energy_vs_oracle(nb, orc):
    s = nb.ics.plummer(2000, seed=9)
    with nb.ScopedParticleData(2000, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                      "mass": s["m"]}) as p:
        pe = nb.Integrator().computePotentialEnergy(p.device, 1.0, 0.01)
    ref = orc.potential_energy(s["x"], s["y"], s["z"], s["m"], 1.0, 0.01)
    assert abs(pe - ref) / abs(ref) < 1e-6


def _c1():
    return 1024, 0.01, 0.001, 100


def test_dropin_trajectory_vs_oracle_fp32(nb, orc):
    n, eps, dt, steps = _c1()
    s = nb.ics.plummer(n, seed=1)
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(eps)
    integ = nb.Integrator()
    arr = {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"], "vel_x": s["vx"],
           "vel_y": s["vy"], "vel_z": s["vz"], "mass": s["m"]}
    with nb.ScopedParticleData(n, arr) as p:
        calc.computeForces(p.device)
        for _ in range(steps):
            integ.integrate(p.device, calc, dt)
        p.download()
        gx, gy, gz = p.host["pos_x"].copy(), p.host["pos_y"].copy(), p.host["pos_z"].copy()
    calc.close()
    # oracle: reference formulas in FP32 with the reference-order direct sum
    x, y, z = s["x"].copy(), s["y"].copy(), s["z"].copy()
    vx, vy, vz = s["vx"].copy(), s["vy"].copy(), s["vz"].copy()
    ax, ay, az = orc.direct_f32(x, y, z, s["m"], 1.0, eps)
    for _ in range(steps):
        ox, oy, oz = ax.copy(), ay.copy(), az.copy()
        orc.update_positions(x, y, z, vx, vy, vz, ax, ay, az, dt)
        ax, ay, az = orc.direct_f32(x, y, z, s["m"], 1.0, eps)
        orc.update_velocities(vx, vy, vz, ox, oy, oz, ax, ay, az, dt)
    dev = max(np.abs(gx - x).max(), np.abs(gy - y).max(), np.abs(gz - z).max())
    assert dev <= 1e-4, dev


def test_system_trajectory_vs_fp64(nb, orc):
    n, eps, dt, steps = _c1()
    s = nb.ics.plummer(n, seed=1)
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(eps)
    sysm = nb.System(calc, s)
    ke0, pe0, _ = sysm.energy()
    sysm.step(dt, steps)
    ke1, pe1, _ = sysm.energy()
    got = sysm.read_f64()
    sysm.close()
    calc.close()
    st = {k: s[k].astype(np.float64) for k in ("x", "y", "z", "vx", "vy", "vz")}
    m = s["m"].astype(np.float64)
    st["ax"], st["ay"], st["az"] = orc.direct_f64(st["x"], st["y"], st["z"], m, 1.0, eps)
    for _ in range(steps):
        orc.vv_step_f64(st, m, 1.0, eps, dt)
    dx = max(np.abs(got[k] - st[k]).max() for k in ("x", "y", "z"))
    dv = max(np.abs(got[k] - st[k]).max() for k in ("vx", "vy", "vz"))
    assert dx <= 2e-5, dx
    assert dv <= 2e-4, dv
    e0, e1 = ke0 + pe0, ke1 + pe1
    assert abs(e1 - e0) / abs(e0) <= 1e-5


def test_system_full_fp64_vs_oracle(nb, orc):
    """NBGB_FLAG_FP64: FP64 forces from the FP64 state.  Trajectory within
    1e-10 of the FP64 oracle after 100 steps (the two differ only in
    summation order and the library rsqrt), energy within 1e-12 relative."""
    n, eps, dt, steps = _c1()
    s = nb.ics.plummer(n, seed=1)
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(eps)
    calc.set_flags(nb.FLAG_SYNC | nb.FLAG_FP64)
    sysm = nb.System(calc, s)
    ke0, pe0, _ = sysm.energy()
    sysm.step(dt, steps)
    got = sysm.read_f64()
    sysm.close()
    calc.close()
    st = {k: s[k].astype(np.float64) for k in ("x", "y", "z", "vx", "vy", "vz")}
    m = s["m"].astype(np.float64)
    eps = float(np.float32(eps))  # the calculator holds softening as a float
    dt = float(np.float32(dt))
    pe_ref = orc.potential_energy(st["x"], st["y"], st["z"], m, 1.0, eps)
    assert abs(pe0 - pe_ref) <= 1e-12 * abs(pe_ref)
    st["ax"], st["ay"], st["az"] = orc.direct_f64(st["x"], st["y"], st["z"], m, 1.0, eps)
    for _ in range(steps):
        orc.vv_step_f64(st, m, 1.0, eps, dt)
    dx = max(np.abs(got[k] - st[k]).max() for k in ("x", "y", "z"))
    dv = max(np.abs(got[k] - st[k]).max() for k in ("vx", "vy", "vz"))
    assert dx <= 1e-10, dx
    assert dv <= 1e-9, dv


def test_fp64_flag_requires_direct(nb):
    s = nb.ics.plummer(256, seed=2)
    calc = nb.BarnesHutCalculator(0.5)
    calc.set_flags(nb.FLAG_SYNC | nb.FLAG_FP64)
    with pytest.raises(nb.ValidationException):
        nb.System(calc, s)
    calc.close()


def test_state_mirror_trajectory_vs_fp64(nb, orc):
    """The drop-in Integrator::integrate path (nbgb_state_kick_drift, the
    calculator, nbgb_state_kick): x and v stay in FP64 inside the library
    between steps.  The plain direct workload, 100 steps: the FP32 ParticleData
    within 2e-5 (x) and 2e-4 (v) of the FP64 oracle's trajectory.  Against
    the device-resident system path (same FP32 forces): after one step the
    FP32 state is the system's FP64 state rounded, bit for bit; after 100
    steps within 5e-6, since the system merges the two half kicks between
    steps into one (v + a dt instead of (v + a dt/2) + a dt/2), which can
    round a position to the neighbouring float, and close pairs amplify
    that."""
    n, eps, dt, steps = _c1()
    s = nb.ics.plummer(n, seed=1)
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(eps)
    integ = nb.Integrator()
    arr = {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"], "vel_x": s["vx"],
           "vel_y": s["vy"], "vel_z": s["vz"], "mass": s["m"]}
    names = (("x", "pos_x"), ("y", "pos_y"), ("z", "pos_z"), ("vx", "vel_x"), ("vy", "vel_y"),
             ("vz", "vel_z"))
    with nb.ScopedParticleData(n, arr) as p:
        calc.computeForces(p.device)
        integ.integrate_f64(p.device, calc, dt)
        p.download()
        one = {k: p.host[f].copy() for k, f in names}
        for _ in range(steps - 1):
            integ.integrate_f64(p.device, calc, dt)
        p.download()
        got = {k: p.host[f].astype(np.float64) for k, f in names}
        integ.release_state(p.device)
    sysm = nb.System(calc, s)
    sysm.step(dt, 1)
    ref1 = sysm.read_f64()
    sysm.close()
    for k, _ in names:
        assert np.array_equal(one[k], ref1[k].astype(np.float32)), k
    st = {k: s[k].astype(np.float64) for k in ("x", "y", "z", "vx", "vy", "vz")}
    m = s["m"].astype(np.float64)
    st["ax"], st["ay"], st["az"] = orc.direct_f64(st["x"], st["y"], st["z"], m, 1.0, eps)
    for _ in range(steps):
        orc.vv_step_f64(st, m, 1.0, eps, float(np.float32(dt)))
    assert max(np.abs(got[k] - st[k]).max() for k in ("x", "y", "z")) <= 2e-5
    assert max(np.abs(got[k] - st[k]).max() for k in ("vx", "vy", "vz")) <= 2e-4
    sysm = nb.System(calc, s)
    sysm.step(dt, steps)
    ref = sysm.read_f64()
    sysm.close()
    calc.close()
    assert max(np.abs(got[k] - ref[k]).max() for k in ("x", "y", "z", "vx", "vy", "vz")) <= 5e-6


def test_state_mirror_takes_caller_changes(nb):
    """A value the caller writes into the FP32 ParticleData between steps (a
    reset, a checkpoint load) becomes the state: the next step starts from it."""
    n, eps, dt = 2000, 0.01, 1e-3
    s = nb.ics.plummer(n, seed=5)
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(eps)
    integ = nb.Integrator()
    arr = {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"], "vel_x": s["vx"],
           "vel_y": s["vy"], "vel_z": s["vz"], "mass": s["m"]}
    with nb.ScopedParticleData(n, arr) as p:
        calc.computeForces(p.device)
        for _ in range(5):
            integ.integrate_f64(p.device, calc, dt)
        p.download()
        p.host["pos_x"][7] += np.float32(0.5)
        p.host["vel_y"][3] = np.float32(0.25)
        p.upload()
        x0, v0 = float(p.host["pos_x"][7]), float(p.host["vel_x"][7])
        a0 = float(p.host["acc_x"][7])
        vy0, ay0 = float(p.host["vel_y"][3]), float(p.host["acc_y"][3])
        integ.integrate_f64(p.device, calc, dt)
        p.download()
        assert abs(p.host["pos_x"][7] - (x0 + v0 * dt + 0.5 * a0 * dt * dt)) <= 1e-6
        ay1 = float(p.host["acc_y"][3])
        assert abs(p.host["vel_y"][3] - (vy0 + 0.5 * (ay0 + ay1) * dt)) <= 1e-6
        integ.release_state(p.device)
    calc.close()


def test_state_mirror_stores_old_accelerations(nb):
    """Each kick-drift leaves acc_old = the acceleration the step started
    from (the reference's storeOldAccelerations), read on the device:
    copyToHost does not copy acc_old (particle_init.cu:148-160)."""
    import torch

    from nbgb.api import FIELDS
    n, eps, dt = 3000, 0.01, 1e-3
    s = nb.ics.plummer(n, seed=6)
    src = {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"], "vel_x": s["vx"],
           "vel_y": s["vy"], "vel_z": s["vz"], "mass": s["m"]}
    dev = {f: torch.from_numpy(np.asarray(src.get(f, np.zeros(n)), np.float32).copy()).cuda()
           for f in FIELDS}
    pd = nb.ParticleData(n)
    pd.on_device = True
    for f in FIELDS:
        setattr(pd.struct, f, dev[f].data_ptr())
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(eps)
    integ = nb.Integrator()
    calc.computeForces(pd)
    for _ in range(3):
        torch.cuda.synchronize()
        a_before = [dev[f].cpu().numpy().copy() for f in ("acc_x", "acc_y", "acc_z")]
        integ.integrate_f64(pd, calc, dt)
        torch.cuda.synchronize()
        for f, a in zip(("acc_old_x", "acc_old_y", "acc_old_z"), a_before):
            np.testing.assert_array_equal(dev[f].cpu().numpy(), a)
    integ.release_state(pd)
    calc.close()
