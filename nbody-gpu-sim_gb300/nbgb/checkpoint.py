"""The reference's `.nbody` v1 checkpoint format (read and written unchanged).

Layout (include/nbody/serialization.hpp:13-32, src/utils/serialization.cpp):
a 56-byte native little-endian header -- u32 magic 0x4E424F44, u32 version 1,
u64 particle_count, f32 simulation_time, dt, G, softening, u32 force_method,
4 x u32 reserved (zero) -- followed by seven contiguous float32 arrays:
pos_x, pos_y, pos_z, vel_x, vel_y, vel_z, mass.  Accelerations are not
stored.  FP64 state is rounded to float32 on save.

The device functions below move the arrays between device memory and the
file through one pinned file image (nbgb_checkpoint_*), and save / load a
device-resident system with an FP64 sidecar <path>.f64 that restores its
exact state (nbgb_system_save / nbgb_system_load).

Load validates like Serializer::load (serialization.cpp:39-75,111-129):
truncated header, wrong magic, unsupported version, count above 1e8,
force method above SPATIAL_HASH and truncated arrays are rejected with the
reference's messages.
"""
from __future__ import annotations

import io
import os
import struct

import numpy as np

from .api import ValidationException

MAGIC = 0x4E424F44
VERSION = 1
MAX_PARTICLE_COUNT = 100_000_000
_HDR = struct.Struct("<IIQffffI4I4x")  # 52 bytes + 4 tail padding (alignof u64)
assert _HDR.size == 56
ARRAYS = ("x", "y", "z", "vx", "vy", "vz", "m")


def save(path_or_file, state: dict, simulation_time: float = 0.0, dt: float = 1e-3,
         G: float = 1.0, softening: float = 0.1, force_method: int = 0) -> None:
    n = len(state["x"])
    hdr = _HDR.pack(MAGIC, VERSION, n, simulation_time, dt, G, softening, int(force_method),
                    0, 0, 0, 0)
    own = isinstance(path_or_file, (str, bytes)) or hasattr(path_or_file, "__fspath__")
    f = open(path_or_file, "wb") if own else path_or_file
    try:
        f.write(hdr)
        for k in ARRAYS:
            a = np.ascontiguousarray(state[k], dtype="<f4")
            if len(a) != n:
                raise ValidationException(f"Validation Error: array {k} length mismatch")
            f.write(a.tobytes())
    finally:
        if own:
            f.close()


def load(path_or_file) -> tuple[dict, dict]:
    """Returns (header dict, arrays dict of float32)."""
    own = isinstance(path_or_file, (str, bytes)) or hasattr(path_or_file, "__fspath__")
    f = open(path_or_file, "rb") if own else path_or_file
    try:
        raw = f.read(56)
        if len(raw) != 56:
            raise ValidationException(
                "Validation Error: Failed to read file header: file may be truncated or corrupted")
        magic, version, n, st, dt, G, eps, method, *_ = _HDR.unpack(raw)
        if magic != MAGIC:
            raise ValidationException("Validation Error: Invalid file format: wrong magic number")
        if version != VERSION:
            raise ValidationException("Validation Error: Unsupported file version")
        if n > MAX_PARTICLE_COUNT:
            raise ValidationException(
                f"Validation Error: Particle count ({n}) exceeds maximum allowed "
                f"({MAX_PARTICLE_COUNT})")
        if method > 2:
            raise ValidationException(
                f"Validation Error: Invalid force method in file header: {method}")
        arrays = {}
        for k in ARRAYS:
            b = f.read(4 * n)
            if len(b) != 4 * n:
                raise ValidationException("Validation Error: Failed to read particle data: "
                                          "file may be truncated or corrupted")
            arrays[k] = np.frombuffer(b, dtype="<f4").astype(np.float32)
        hdr = dict(particle_count=n, simulation_time=st, dt=dt, G=G, softening=eps,
                   force_method=method)
        return hdr, arrays
    finally:
        if own:
            f.close()


def to_bytes(state: dict, **kw) -> bytes:
    b = io.BytesIO()
    save(b, state, **kw)
    return b.getvalue()


# --- device fast path (nbgb_checkpoint_*, nbgb_system_save / load) -----------
def _hdr(simulation_time=0.0, dt=1e-3, G=1.0, softening=0.1, force_method=0):
    from ._lib import CheckpointHeader
    h = CheckpointHeader()
    h.simulation_time, h.dt, h.G, h.softening = simulation_time, dt, G, softening
    h.force_method = int(force_method)
    return h


def _header_dict(h) -> dict:
    return dict(particle_count=h.particle_count, simulation_time=h.simulation_time, dt=h.dt,
                G=h.G, softening=h.softening, force_method=h.force_method)


def save_device(path, d, **header) -> None:
    """The v1 file of device ParticleData `d` (pos, vel, mass), written from one
    pinned file image (the same bytes as save() of the same float32 arrays)."""
    import ctypes as C

    from . import _lib
    from .api import check
    h = _hdr(**header)
    check(_lib.lib().nbgb_checkpoint_save_device(os.fsencode(path), d.ptr(), C.byref(h), None))


def load_device(path, d) -> dict:
    """Reads a v1 file into device ParticleData `d` (count must match); returns
    the header.  With d None, reads the header only."""
    import ctypes as C

    from . import _lib
    from ._lib import CheckpointHeader
    from .api import check
    h = CheckpointHeader()
    check(_lib.lib().nbgb_checkpoint_load_device(os.fsencode(path), d.ptr() if d else None,
                                                 C.byref(h), None))
    return _header_dict(h)


def save_system(path, system, with_f64: bool = True, **header) -> None:
    """A device-resident system's state as v1 (+ the FP64 sidecar <path>.f64)."""
    import ctypes as C

    from . import _lib
    from .api import check
    h = _hdr(**header)
    check(_lib.lib().nbgb_system_save(system.handle, os.fsencode(path), C.byref(h),
                                      1 if with_f64 else 0))


def load_system(path, calc):
    """(System, header dict, FP64 state restored?) from a checkpoint."""
    import ctypes as C

    from . import _lib
    from ._lib import CheckpointHeader
    from .api import System, check
    h = CheckpointHeader()
    hd = C.c_void_p()
    restored = C.c_int32(0)
    check(_lib.lib().nbgb_system_load(calc.handle, os.fsencode(path), C.byref(hd), C.byref(h),
                                      C.byref(restored)))
    sysm = System.__new__(System)
    sysm.calc, sysm.n, sysm.handle = calc, int(h.particle_count), hd
    return sysm, _header_dict(h), bool(restored.value)
