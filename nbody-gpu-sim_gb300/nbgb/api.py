"""Host-side mirror of the reference's `include/nbody` hot-path interface.

Same class and method names as the reference (ForceCalculator and its
subclasses, createForceCalculator, Integrator, ParticleDataManager), same
argument meaning, and the same exception kinds, implemented over the C ABI
of libnbgb.so.  Device particle data is a `ParticleData` struct of 13 device
pointers (nbody::ParticleData layout); host data is a dict of numpy arrays.
"""
from __future__ import annotations

import ctypes as C
from enum import IntEnum

import numpy as np

from . import _lib
from ._lib import (FLAG_COMPENSATED, FLAG_COUNT_INTERACTIONS, FLAG_FP64, FLAG_GROUP_WALK,
                   FLAG_REFERENCE_TREE, FLAG_STAGE_TIMINGS, FLAG_SYNC, OctreeNode, Params)
from ._lib import ParticleDataStruct

FIELDS = ("pos_x", "pos_y", "pos_z", "vel_x", "vel_y", "vel_z", "acc_x", "acc_y", "acc_z",
          "acc_old_x", "acc_old_y", "acc_old_z", "mass")


class ForceMethod(IntEnum):
    """== nbody::ForceMethod (include/nbody/types.hpp:35)."""
    DIRECT_N2 = 0
    BARNES_HUT = 1
    SPATIAL_HASH = 2


def forceMethodToString(m: ForceMethod) -> str:  # noqa: N802  (types.hpp:39-49)
    return {ForceMethod.DIRECT_N2: "direct_n2", ForceMethod.BARNES_HUT: "barnes_hut",
            ForceMethod.SPATIAL_HASH: "spatial_hash"}.get(ForceMethod(m), "unknown")


# -- exceptions (include/nbody/error_handling.hpp) ----------------------------
class NbodyError(RuntimeError):
    status = -1


class ValidationException(NbodyError):
    """include/nbody/error_handling.hpp:98-102 ("Validation Error: ...")."""


class ResourceException(NbodyError):
    """include/nbody/error_handling.hpp:76-95."""


class CudaException(NbodyError):
    """include/nbody/error_handling.hpp:29-51 ("CUDA Error: ...")."""


class DeviceTimeout(NbodyError):
    """A bounded device-side wait ran out (the kernel returned an error word)."""


class CapacityError(NbodyError):
    """Spatial-hash grid above 1e8 cells (force_spatial_hash.cu:258-260) or a
    device capacity exceeded."""


_STATUS = {1: ValidationException, 2: ResourceException, 3: CudaException, 4: DeviceTimeout,
           5: CapacityError, 6: NbodyError, 7: CudaException}


def check(status: int) -> None:
    if status != 0:
        msg = _lib.lib().nbgb_last_error().decode(errors="replace")
        exc = _STATUS.get(status, NbodyError)(msg or f"nbgb status {status}")
        exc.status = status
        raise exc


# -- particle data --------------------------------------------------------------
class ParticleData:
    """A ParticleData struct (13 pointers + count) viewed from Python.

    `ParticleData.host(arrays)` wraps host numpy arrays (kept alive by the
    object); `ParticleDataManager.allocateDevice(n)` returns a device one.
    """

    def __init__(self, count: int = 0) -> None:
        self.struct = ParticleDataStruct()
        self.struct.count = count
        self.on_device = False
        self._keep: dict[str, np.ndarray] = {}

    @property
    def count(self) -> int:
        return int(self.struct.count)

    @classmethod
    def host(cls, arrays: dict[str, np.ndarray] | None = None, count: int | None = None):
        """Host SoA; missing fields are zero-filled (acc/acc_old default 0)."""
        arrays = dict(arrays or {})
        n = count if count is not None else len(next(iter(arrays.values())))
        pd = cls(n)
        for f in FIELDS:
            a = arrays.get(f)
            # always a private copy: downloads must never write into caller arrays
            a = np.zeros(n, np.float32) if a is None else np.array(a, dtype=np.float32, copy=True)
            if len(a) != n:
                raise ValidationException(f"Validation Error: field {f} has length {len(a)} != {n}")
            pd._keep[f] = a
            setattr(pd.struct, f, a.ctypes.data if n else None)
        return pd

    def array(self, field: str) -> np.ndarray:
        if self.on_device:
            raise ValueError("device data: use ParticleDataManager.copyToHost")
        return self._keep[field]

    def ptr(self):
        return C.byref(self.struct)

    def __getitem__(self, field: str) -> np.ndarray:
        return self.array(field)


class ParticleDataManager:
    """include/nbody/particle_data.hpp:9-28."""

    @staticmethod
    def allocateDevice(count: int) -> ParticleData:  # noqa: N802
        pd = ParticleData(count)
        check(_lib.lib().nbgb_particles_alloc_device(pd.ptr(), count))
        pd.on_device = True
        return pd

    @staticmethod
    def freeDevice(pd: ParticleData) -> None:  # noqa: N802
        if pd.on_device:
            check(_lib.lib().nbgb_particles_free_device(pd.ptr()))
            pd.on_device = False

    @staticmethod
    def copyToDevice(d: ParticleData, h: ParticleData) -> None:  # noqa: N802
        check(_lib.lib().nbgb_particles_copy_to_device(d.ptr(), h.ptr()))

    @staticmethod
    def copyToHost(h: ParticleData, d: ParticleData) -> None:  # noqa: N802
        check(_lib.lib().nbgb_particles_copy_to_host(h.ptr(), d.ptr()))

    @staticmethod
    def initDevice(d: ParticleData, distribution: int, seed: int = 42,  # noqa: N802
                   **params) -> None:
        """Initial conditions generated in the device arrays of d
        (nbgb_init_particles_device); params override the defaults of
        nbgb_init_params_default (center, radius, min_bounds, max_bounds,
        min_mass, max_mass, thickness, rotation_speed, plummer_a,
        total_mass, G)."""
        p = _lib.InitParams()
        _lib.lib().nbgb_init_params_default(C.byref(p), distribution)
        for k, v in params.items():
            if k in ("center", "min_bounds", "max_bounds"):
                getattr(p, k)[:] = [float(x) for x in v]
            else:
                setattr(p, k, v)
        check(_lib.lib().nbgb_init_particles_device(d.ptr(), C.byref(p), seed, None))


class ScopedParticleData:
    """Device + host pair, like tests/particle_data_fixture.hpp:11-27."""

    def __init__(self, count: int, arrays: dict[str, np.ndarray] | None = None) -> None:
        self.host = ParticleData.host(arrays, count=count)
        self.device = ParticleDataManager.allocateDevice(count)
        if arrays:
            self.upload()

    def upload(self) -> None:
        ParticleDataManager.copyToDevice(self.device, self.host)

    def download(self) -> None:
        ParticleDataManager.copyToHost(self.host, self.device)

    def close(self) -> None:
        ParticleDataManager.freeDevice(self.device)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# -- force calculators (include/nbody/force_calculator.hpp) ---------------------
def default_params() -> Params:
    p = Params()
    _lib.lib().nbgb_params_default(C.byref(p))
    return p


class ForceCalculator:
    """include/nbody/force_calculator.hpp:8-27 over an nbgb_calculator handle."""

    method: ForceMethod = ForceMethod.DIRECT_N2

    def __init__(self, params: Params | None = None) -> None:
        self._p = params if params is not None else default_params()
        h = C.c_void_p()
        check(_lib.lib().nbgb_calculator_create(int(self.method), C.byref(self._p), C.byref(h)))
        self.handle = h

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.lib().nbgb_calculator_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _apply(self) -> None:
        check(_lib.lib().nbgb_calculator_set_params(self.handle, C.byref(self._p)))

    # reference API
    def computeForces(self, d: ParticleData) -> None:  # noqa: N802
        check(_lib.lib().nbgb_compute_forces(self.handle, d.ptr()))

    def getMethod(self) -> ForceMethod:  # noqa: N802
        return self.method

    def setSofteningParameter(self, eps: float) -> None:  # noqa: N802
        self._p.softening = eps
        self._apply()

    def setGravitationalConstant(self, G: float) -> None:  # noqa: N802,N803
        self._p.G = G
        self._apply()

    def getSofteningParameter(self) -> float:  # noqa: N802
        return float(self._p.softening)

    def getGravitationalConstant(self) -> float:  # noqa: N802
        return float(self._p.G)

    # library extensions
    @property
    def params(self) -> Params:
        return self._p

    def set_flags(self, flags: int) -> None:
        self._p.flags = flags
        self._apply()

    def set_stream(self, stream_handle: int | None) -> None:
        check(_lib.lib().nbgb_calculator_set_stream(self.handle, C.c_void_p(stream_handle or 0)))

    def synchronize(self) -> None:
        check(_lib.lib().nbgb_calculator_synchronize(self.handle))

    def stage_times(self, reset: bool = False) -> dict[str, tuple[float, int]]:
        """Device milliseconds and run count per stage of the force evaluations
        made with FLAG_STAGE_TIMINGS (nbgb_calculator_stage_times)."""
        cap = 32
        names = C.create_string_buffer(32 * cap)
        ms = (C.c_double * cap)()
        cnt = (C.c_int64 * cap)()
        k = C.c_int32(0)
        check(_lib.lib().nbgb_calculator_stage_times(self.handle, cap, names, ms, cnt,
                                                     C.byref(k), int(reset)))
        raw = names.raw
        return {raw[32 * i:32 * i + 32].split(b"\0")[0].decode(): (ms[i], cnt[i])
                for i in range(min(k.value, cap))}

    def interaction_counts(self, n: int) -> np.ndarray:
        out = np.zeros(n, np.int32)
        check(_lib.lib().nbgb_copy_interaction_counts(self.handle, out.ctypes.data, n))
        return out


class DirectForceCalculator(ForceCalculator):
    """force_calculator.hpp:29-39."""
    method = ForceMethod.DIRECT_N2

    def __init__(self, block_size: int = 256, params: Params | None = None) -> None:
        p = params if params is not None else default_params()
        p.block_size = block_size
        super().__init__(p)

    def setBlockSize(self, size: int) -> None:  # noqa: N802
        self._p.block_size = size
        self._apply()

    def getBlockSize(self) -> int:  # noqa: N802
        return int(self._p.block_size)


class BarnesHutCalculator(ForceCalculator):
    """force_calculator.hpp:41-54 (leaf_capacity=1 is the reference tree)."""
    method = ForceMethod.BARNES_HUT

    def __init__(self, theta: float = 0.5, leaf_capacity: int = 1,
                 params: Params | None = None, group_walk: bool = False,
                 group_size: int = 0) -> None:
        """group_size: the group walk's largest group (32 or 64; 0 = by the
        body count, as nbgb_bh_group_size)."""
        p = params if params is not None else default_params()
        p.theta = theta
        p.leaf_capacity = leaf_capacity
        p.group_size = group_size
        if group_walk:
            p.flags |= FLAG_GROUP_WALK
        super().__init__(p)

    def setTheta(self, theta: float) -> None:  # noqa: N802
        self._p.theta = theta
        self._apply()

    def getTheta(self) -> float:  # noqa: N802
        return float(self._p.theta)

    # BarnesHutTree inspection (barnes_hut_tree.hpp:55-65)
    def tree_stats(self) -> tuple[int, int]:
        nc, md = C.c_int32(0), C.c_int32(0)
        check(_lib.lib().nbgb_bh_tree_stats(self.handle, C.byref(nc), C.byref(md)))
        return nc.value, md.value

    def sorted_keys(self, n: int) -> tuple[np.ndarray, np.ndarray]:
        k = np.zeros(n, np.uint32)
        v = np.zeros(n, np.int32)
        check(_lib.lib().nbgb_bh_copy_sorted_keys(self.handle, k.ctypes.data, v.ctypes.data, n))
        return k, v

    def nodes(self) -> np.ndarray:
        from .layout import NODE_DTYPE
        nc, _ = self.tree_stats()
        out = np.zeros(max(nc, 1), NODE_DTYPE)
        check(_lib.lib().nbgb_bh_copy_nodes(self.handle, out.ctypes.data, len(out)))
        return out[:nc]


class SpatialHashCalculator(ForceCalculator):
    """force_calculator.hpp:56-74."""
    method = ForceMethod.SPATIAL_HASH

    def __init__(self, cell_size: float = 2.0, cutoff_radius: float = 2.0,
                 params: Params | None = None) -> None:
        p = params if params is not None else default_params()
        p.cell_size = cell_size
        p.cutoff = cutoff_radius
        super().__init__(p)

    def setCellSize(self, size: float) -> None:  # noqa: N802
        self._p.cell_size = size
        self._apply()

    def setCutoffRadius(self, r: float) -> None:  # noqa: N802
        self._p.cutoff = r
        self._apply()

    def getCellSize(self) -> float:  # noqa: N802
        return float(self._p.cell_size)

    def getCutoffRadius(self) -> float:  # noqa: N802
        return float(self._p.cutoff)

    # SpatialHashGrid inspection (spatial_hash_grid.hpp:25-31)
    def grid_info(self) -> dict:
        dims = (C.c_int32 * 3)()
        bmin = (C.c_float * 3)()
        cell = C.c_float(0)
        tot = C.c_int64(0)
        check(_lib.lib().nbgb_hash_grid_info(self.handle, dims, bmin, C.byref(cell), C.byref(tot)))
        return dict(dims=np.array(list(dims), np.int32), bmin=np.array(list(bmin), np.float32),
                    cell=np.float32(cell.value), total_cells=tot.value)

    def cell_data(self, n: int) -> dict:
        info = self.grid_info()
        tot = info["total_cells"]
        cs = np.zeros(tot, np.int32)
        ce = np.zeros(tot, np.int32)
        pc = np.zeros(n, np.int32)
        si = np.zeros(n, np.int32)
        check(_lib.lib().nbgb_hash_copy_cells(self.handle, cs.ctypes.data, ce.ctypes.data,
                                               pc.ctypes.data, si.ctypes.data))
        info.update(cell_start=cs, cell_end=ce, particle_cell=pc, sorted_indices=si)
        return info


def createForceCalculator(method: ForceMethod, config: dict | None = None) -> ForceCalculator:  # noqa: N802
    """createForceCalculator (force_spatial_hash.cu:391-404) from a
    SimulationConfig-like dict (types.hpp:133-144 keys)."""
    cfg = dict(cuda_block_size=256, barnes_hut_theta=0.5, spatial_hash_cell_size=2.0,
               spatial_hash_cutoff=2.0)
    cfg.update(config or {})
    m = ForceMethod(method)
    if m == ForceMethod.BARNES_HUT:
        return BarnesHutCalculator(cfg["barnes_hut_theta"])
    if m == ForceMethod.SPATIAL_HASH:
        return SpatialHashCalculator(cfg["spatial_hash_cell_size"], cfg["spatial_hash_cutoff"])
    return DirectForceCalculator(cfg["cuda_block_size"])


# -- integrator (include/nbody/integrator.hpp) ----------------------------------
class Integrator:
    """integrator.hpp:15-33; energies are FP64 reductions returned as float."""

    def __init__(self, block_size: int = 256) -> None:
        self.block_size = block_size

    def integrate(self, d: ParticleData, calc: ForceCalculator, dt: float) -> None:
        """The reference's FP32 update kernels around the forces (integrator.cu:175-189)."""
        check(_lib.lib().nbgb_integrate(calc.handle, d.ptr(), dt))

    def integrate_f64(self, d: ParticleData, calc: ForceCalculator, dt: float) -> None:
        """The same step with x and v kept in FP64 by the library between steps
        (the drop-in adapter's Integrator::integrate); d holds the rounded state."""
        check(_lib.lib().nbgb_state_kick_drift(d.ptr(), dt, None))
        calc.computeForces(d)
        check(_lib.lib().nbgb_state_kick(d.ptr(), dt, None))

    def release_state(self, d: ParticleData) -> None:
        check(_lib.lib().nbgb_state_release(d.ptr()))

    def updatePositions(self, d: ParticleData, dt: float) -> None:  # noqa: N802
        check(_lib.lib().nbgb_update_positions(d.ptr(), dt, None))

    def updateVelocities(self, d: ParticleData, dt: float) -> None:  # noqa: N802
        check(_lib.lib().nbgb_update_velocities(d.ptr(), dt, None))

    def storeOldAccelerations(self, d: ParticleData) -> None:  # noqa: N802
        check(_lib.lib().nbgb_store_old_accelerations(d.ptr(), None))

    def computeKineticEnergy(self, d: ParticleData) -> float:  # noqa: N802
        v = C.c_double(0)
        check(_lib.lib().nbgb_kinetic_energy(d.ptr(), C.byref(v), None))
        return v.value

    def computePotentialEnergy(self, d: ParticleData, G: float, eps: float) -> float:  # noqa: N802,N803
        v = C.c_double(0)
        check(_lib.lib().nbgb_potential_energy(d.ptr(), G, eps, C.byref(v), None))
        return v.value

    def computeTotalEnergy(self, d: ParticleData, G: float, eps: float) -> float:  # noqa: N802,N803
        return self.computeKineticEnergy(d) + self.computePotentialEnergy(d, G, eps)


# -- device-resident FP64 system ------------------------------------------------
class System:
    """nbgb_system: FP64 x/v state on the device, FP32 forces from `calc`."""

    def __init__(self, calc: ForceCalculator, state: dict[str, np.ndarray]) -> None:
        self.calc = calc
        n = len(state["x"])
        self.n = n
        h = ParticleData.host({"pos_x": state["x"], "pos_y": state["y"], "pos_z": state["z"],
                               "vel_x": state["vx"], "vel_y": state["vy"], "vel_z": state["vz"],
                               "mass": state["m"]})
        hd = C.c_void_p()
        check(_lib.lib().nbgb_system_create(calc.handle, h.ptr(), C.byref(hd)))
        self.handle = hd

    def step(self, dt: float, steps: int = 1) -> None:
        check(_lib.lib().nbgb_system_step(self.handle, dt, steps))

    def read(self) -> dict[str, np.ndarray]:
        h = ParticleData.host(count=self.n)
        check(_lib.lib().nbgb_system_read(self.handle, h.ptr()))
        return {k: h.array(f) for k, f in (("x", "pos_x"), ("y", "pos_y"), ("z", "pos_z"),
                                           ("vx", "vel_x"), ("vy", "vel_y"), ("vz", "vel_z"),
                                           ("ax", "acc_x"), ("ay", "acc_y"), ("az", "acc_z"),
                                           ("m", "mass"))}

    def read_f64(self) -> dict[str, np.ndarray]:
        out = {k: np.zeros(self.n, np.float64) for k in ("x", "y", "z", "vx", "vy", "vz")}
        check(_lib.lib().nbgb_system_read_f64(self.handle, *[out[k].ctypes.data for k in
                                                             ("x", "y", "z", "vx", "vy", "vz")]))
        return out

    def energy(self) -> tuple[float, float, np.ndarray]:
        ke, pe = C.c_double(0), C.c_double(0)
        mom = (C.c_double * 3)()
        check(_lib.lib().nbgb_system_energy(self.handle, C.byref(ke), C.byref(pe), mom))
        return ke.value, pe.value, np.array(list(mom))

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.lib().nbgb_system_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["ForceMethod", "forceMethodToString", "ParticleData", "ParticleDataManager",
           "ScopedParticleData", "ForceCalculator", "DirectForceCalculator",
           "BarnesHutCalculator", "SpatialHashCalculator", "createForceCalculator",
           "Integrator", "System", "ValidationException", "ResourceException", "CudaException",
           "DeviceTimeout", "CapacityError", "NbodyError", "check", "default_params",
           "FLAG_SYNC", "FLAG_COMPENSATED", "FLAG_COUNT_INTERACTIONS", "FLAG_FP64", "FLAG_GROUP_WALK",
           "FLAG_REFERENCE_TREE", "FLAG_STAGE_TIMINGS",
           "OctreeNode",
           "Params"]
