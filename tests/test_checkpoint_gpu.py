"""Checkpoints from and into device memory (GPU).

* The device writer's v1 file is byte-identical to the host writer's
  (nbgb.checkpoint.save, itself byte-identical to the reference's
  Serializer::save: tests/test_checkpoint.py) and reads back into device
  memory unchanged; the reference-written golden file loads too.
* A device-resident system saved with the FP64 sidecar and loaded again
  continues bitwise as the saved system does; without the sidecar it
  continues from the float32 state.
* Load errors carry the reference's messages.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _arrays(s):
    return {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"], "vel_x": s["vx"],
            "vel_y": s["vy"], "vel_z": s["vz"], "mass": s["m"]}


def test_device_v1_equals_host_writer_and_round_trips(nb, tmp_path):
    from nbgb import checkpoint as ck
    s = nb.ics.plummer(5000, seed=61)
    hdr = dict(simulation_time=1.5, dt=2e-3, G=1.25, softening=0.05, force_method=1)
    with nb.ScopedParticleData(5000, _arrays(s)) as p:
        ck.save_device(tmp_path / "dev.nbody", p.device, **hdr)
    ck.save(tmp_path / "host.nbody", s, **hdr)
    assert (tmp_path / "dev.nbody").read_bytes() == (tmp_path / "host.nbody").read_bytes()
    assert ck.load_device(tmp_path / "dev.nbody", None)["particle_count"] == 5000
    with nb.ScopedParticleData(5000) as q:
        got = ck.load_device(tmp_path / "dev.nbody", q.device)
        q.download()
        for k, f in (("x", "pos_x"), ("vy", "vel_y"), ("m", "mass")):
            np.testing.assert_array_equal(q.host[f], s[k])
    assert got["force_method"] == 1 and abs(got["G"] - 1.25) < 1e-7


def test_reference_golden_file_loads_on_device(nb):
    import os

    from conftest import GOLDEN
    from nbgb import checkpoint as ck
    path = os.path.join(GOLDEN, "ref_checkpoint.nbody")
    hdr, arr = ck.load(path)
    n = hdr["particle_count"]
    with nb.ScopedParticleData(n) as q:
        got = ck.load_device(path, q.device)
        q.download()
        np.testing.assert_array_equal(q.host["vel_x"], arr["vx"])
    assert got["force_method"] == hdr["force_method"]


def test_system_restart_is_bitwise_with_fp64_sidecar(nb, tmp_path):
    from nbgb import checkpoint as ck
    s = nb.ics.plummer(3000, seed=62)
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(0.01)
    a = nb.System(calc, s)
    a.step(1e-3, 30)
    ck.save_system(tmp_path / "run.nbody", a, simulation_time=0.03, dt=1e-3, softening=0.01)
    a.step(1e-3, 30)
    ref = a.read_f64()
    a.close()
    b, hdr, restored = ck.load_system(tmp_path / "run.nbody", calc)
    assert restored and hdr["particle_count"] == 3000
    b.step(1e-3, 30)
    got = b.read_f64()
    b.close()
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        np.testing.assert_array_equal(got[k], ref[k])
    # without the sidecar the run continues from the float32 state
    (tmp_path / "run.nbody.f64").unlink()
    c, _, restored = ck.load_system(tmp_path / "run.nbody", calc)
    assert not restored
    c.step(1e-3, 30)
    got32 = c.read_f64()
    c.close()
    calc.close()
    assert max(np.abs(got32[k] - ref[k]).max() for k in ("x", "y", "z")) <= 1e-5


def test_load_errors_carry_reference_messages(nb, tmp_path):
    from nbgb import checkpoint as ck
    bad = tmp_path / "bad.nbody"
    bad.write_bytes(b"\x00" * 10)
    with pytest.raises(nb.ValidationException, match="truncated or corrupted"):
        ck.load_device(bad, None)
    raw = bytearray(ck.to_bytes(nb.ics.plummer(10, seed=1)))
    raw[0] ^= 0xFF
    bad.write_bytes(bytes(raw))
    with pytest.raises(nb.ValidationException, match="wrong magic number"):
        ck.load_device(bad, None)
