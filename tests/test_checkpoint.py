"""`.nbody` v1 checkpoint format against the reference's Serializer
(tests/test_serialization.cpp restated).  CPU only."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import GOLDEN


def _state(n=5, seed=0):
    rng = np.random.default_rng(seed)
    return {k: rng.normal(size=n).astype(np.float32) for k in ("x", "y", "z", "vx", "vy", "vz", "m")}


def test_reads_reference_written_file(nb):
    hdr, arr = nb.checkpoint.load(os.path.join(GOLDEN, "ref_checkpoint.nbody"))
    assert hdr["particle_count"] == 7 and hdr["force_method"] == 2
    assert hdr["simulation_time"] == pytest.approx(1.25) and hdr["dt"] == pytest.approx(0.002)
    assert hdr["G"] == pytest.approx(1.5) and hdr["softening"] == pytest.approx(0.05)
    np.testing.assert_allclose(arr["vx"], np.linspace(-1, 1, 7).astype(np.float32))


def test_writes_reference_bytes(nb):
    path = os.path.join(GOLDEN, "ref_checkpoint.nbody")
    hdr, arr = nb.checkpoint.load(path)
    again = nb.checkpoint.to_bytes(arr, simulation_time=hdr["simulation_time"], dt=hdr["dt"],
                                   G=hdr["G"], softening=hdr["softening"],
                                   force_method=hdr["force_method"])
    assert again == open(path, "rb").read()


def test_round_trip(nb, tmp_path):
    s = _state(100)
    p = tmp_path / "a.nbody"
    nb.checkpoint.save(p, s, simulation_time=3.0, dt=0.01, G=2.0, softening=0.2, force_method=1)
    hdr, arr = nb.checkpoint.load(p)
    assert hdr["particle_count"] == 100 and hdr["force_method"] == 1
    for k in s:
        np.testing.assert_array_equal(arr[k], s[k])
    assert os.path.getsize(p) == 56 + 7 * 4 * 100


@pytest.mark.parametrize("mutate,msg", [
    (lambda b: b[:40], "header"),
    (lambda b: b"\0\0\0\0" + b[4:], "magic"),
    (lambda b: b[:4] + (2).to_bytes(4, "little") + b[8:], "version"),
    (lambda b: b[:8] + (100_000_001).to_bytes(8, "little") + b[16:], "exceeds maximum"),
    (lambda b: b[:32] + (3).to_bytes(4, "little") + b[36:], "force method"),
    (lambda b: b[:-4], "particle data"),
])
def test_rejections(nb, tmp_path, mutate, msg):
    # tests/test_serialization.cpp:153-195
    good = nb.checkpoint.to_bytes(_state(4))
    p = tmp_path / "bad.nbody"
    p.write_bytes(mutate(good))
    with pytest.raises(nb.ValidationException, match=msg):
        nb.checkpoint.load(p)
