"""ctypes binding of libnbgb.so (the C ABI declared in include/nbgb.h).

Loading this module loads the CUDA library; it fails loudly when the library
is missing (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import build as _build

_HEADER = os.path.join(_build.REPO, "include", "nbgb.h")


class Params(C.Structure):
    _fields_ = [("G", C.c_float), ("softening", C.c_float), ("theta", C.c_float),
                ("cell_size", C.c_float), ("cutoff", C.c_float), ("block_size", C.c_int32),
                ("leaf_capacity", C.c_int32), ("flags", C.c_uint32), ("group_size", C.c_int32)]


class ParticleDataStruct(C.Structure):
    """== nbgb_particle_data == nbody::ParticleData (13 float* + size_t)."""
    _fields_ = [(name, C.c_void_p) for name in (
        "pos_x", "pos_y", "pos_z", "vel_x", "vel_y", "vel_z", "acc_x", "acc_y", "acc_z",
        "acc_old_x", "acc_old_y", "acc_old_z", "mass")] + [("count", C.c_size_t)]


class OctreeNode(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("half_size", C.c_float),
                ("center_of_mass", C.c_float * 3), ("total_mass", C.c_float),
                ("children", C.c_int32 * 8), ("particle_index", C.c_int32),
                ("is_leaf", C.c_uint8), ("pad_", C.c_uint8 * 3), ("particle_count", C.c_int32)]


class InitParams(C.Structure):
    _fields_ = [("distribution", C.c_int32), ("center", C.c_float * 3), ("radius", C.c_float),
                ("min_bounds", C.c_float * 3), ("max_bounds", C.c_float * 3),
                ("min_mass", C.c_float), ("max_mass", C.c_float), ("thickness", C.c_float),
                ("rotation_speed", C.c_float), ("plummer_a", C.c_float),
                ("total_mass", C.c_float), ("G", C.c_float)]


DIST_UNIFORM, DIST_SPHERICAL, DIST_DISK, DIST_PLUMMER = 0, 1, 2, 3


class EnsembleConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_resident", C.c_int32),
                ("direct_max_n", C.c_int32), ("G", C.c_float), ("softening", C.c_float),
                ("theta", C.c_float), ("leaf_capacity", C.c_int32), ("direct_config", C.c_int32),
                ("use_graphs", C.c_int32), ("group_walk", C.c_int32)]


class EnsembleResult(C.Structure):
    _fields_ = [("request_id", C.c_uint64), ("count", C.c_int64), ("steps", C.c_int32),
                ("method", C.c_int32), ("gpu_ms", C.c_double)]


class CheckpointHeader(C.Structure):
    _fields_ = [("particle_count", C.c_uint64), ("simulation_time", C.c_float),
                ("dt", C.c_float), ("G", C.c_float), ("softening", C.c_float),
                ("force_method", C.c_uint32)]


class EnsembleStats(C.Structure):
    _fields_ = [("ticks", C.c_int64), ("particle_steps", C.c_int64),
                ("direct_interactions", C.c_double), ("bh_interactions", C.c_double),
                ("admitted", C.c_int64), ("retired", C.c_int64), ("resident", C.c_int32),
                ("queued", C.c_int32), ("bytes_reserved", C.c_uint64),
                ("direct_config", C.c_int32), ("tuning", C.c_int32),
                ("direct_kernel_ms", C.c_double), ("direct_kernel_interactions", C.c_double),
                ("kernel_launches", C.c_int64), ("bh_walk_ms", C.c_double),
                ("bh_bodies", C.c_int64)]


assert C.sizeof(OctreeNode) == 76
assert C.sizeof(ParticleDataStruct) == 13 * 8 + 8

FLAG_SYNC = 0x1
FLAG_COMPENSATED = 0x2
FLAG_COUNT_INTERACTIONS = 0x4
FLAG_FP64 = 0x8
FLAG_GROUP_WALK = 0x10
FLAG_REFERENCE_TREE = 0x20
FLAG_STAGE_TIMINGS = 0x40

_vp = C.c_void_p
_i32p = C.POINTER(C.c_int32)
_u32p = C.POINTER(C.c_uint32)
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_pd = C.POINTER(ParticleDataStruct)

# name -> (restype, argtypes)
_SIGS = {
    "nbgb_params_default": (None, [C.POINTER(Params)]),
    "nbgb_calculator_create": (C.c_int, [C.c_int, C.POINTER(Params), C.POINTER(_vp)]),
    "nbgb_calculator_destroy": (C.c_int, [_vp]),
    "nbgb_calculator_set_params": (C.c_int, [_vp, C.POINTER(Params)]),
    "nbgb_calculator_get_params": (C.c_int, [_vp, C.POINTER(Params)]),
    "nbgb_calculator_get_method": (C.c_int, [_vp, C.POINTER(C.c_int)]),
    "nbgb_calculator_set_stream": (C.c_int, [_vp, _vp]),
    "nbgb_calculator_synchronize": (C.c_int, [_vp]),
    "nbgb_calculator_stage_times": (C.c_int, [_vp, C.c_int32, C.c_char_p,
                                              C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                              C.POINTER(C.c_int32), C.c_int32]),
    "nbgb_compute_forces": (C.c_int, [_vp, _pd]),
    "nbgb_integrate": (C.c_int, [_vp, _pd, C.c_float]),
    "nbgb_state_kick_drift": (C.c_int, [_pd, C.c_float, _vp]),
    "nbgb_state_kick": (C.c_int, [_pd, C.c_float, _vp]),
    "nbgb_state_release": (C.c_int, [_pd]),
    "nbgb_update_positions": (C.c_int, [_pd, C.c_float, _vp]),
    "nbgb_update_velocities": (C.c_int, [_pd, C.c_float, _vp]),
    "nbgb_store_old_accelerations": (C.c_int, [_pd, _vp]),
    "nbgb_kinetic_energy": (C.c_int, [_pd, _f64p, _vp]),
    "nbgb_potential_energy": (C.c_int, [_pd, C.c_float, C.c_float, _f64p, _vp]),
    "nbgb_particles_alloc_device": (C.c_int, [_pd, C.c_size_t]),
    "nbgb_particles_free_device": (C.c_int, [_pd]),
    "nbgb_particles_copy_to_device": (C.c_int, [_pd, _pd]),
    "nbgb_particles_copy_to_host": (C.c_int, [_pd, _pd]),
    "nbgb_init_params_default": (None, [C.POINTER(InitParams), C.c_int32]),
    "nbgb_selftest_wait_timeout": (C.c_int, [C.c_uint32, C.POINTER(C.c_uint32)]),
    "nbgb_selftest_group_walk_stack": (C.c_int, [C.c_int32]),
    "nbgb_selftest_fail_allocation": (C.c_int, [C.c_int32]),
    "nbgb_bh_group_size": (C.c_int32, [C.c_uint64]),
    "nbgb_init_particles_device": (C.c_int, [_pd, C.POINTER(InitParams), C.c_uint64, _vp]),
    "nbgb_bh_tree_stats": (C.c_int, [_vp, _i32p, _i32p]),
    "nbgb_bh_copy_sorted_keys": (C.c_int, [_vp, _vp, _vp, C.c_size_t]),
    "nbgb_bh_copy_nodes": (C.c_int, [_vp, _vp, C.c_size_t]),
    "nbgb_hash_grid_info": (C.c_int, [_vp, _i32p, _f32p, _f32p, C.POINTER(C.c_int64)]),
    "nbgb_hash_copy_cells": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "nbgb_copy_interaction_counts": (C.c_int, [_vp, _vp, C.c_size_t]),
    "nbgb_system_create": (C.c_int, [_vp, _pd, C.POINTER(_vp)]),
    "nbgb_system_destroy": (C.c_int, [_vp]),
    "nbgb_system_step": (C.c_int, [_vp, C.c_float, C.c_int32]),
    "nbgb_system_read": (C.c_int, [_vp, _pd]),
    "nbgb_system_read_f64": (C.c_int, [_vp] + [_vp] * 6),
    "nbgb_system_energy": (C.c_int, [_vp, _f64p, _f64p, _f64p]),
    "nbgb_checkpoint_save_device": (C.c_int, [C.c_char_p, _pd, C.POINTER(CheckpointHeader), _vp]),
    "nbgb_checkpoint_load_device": (C.c_int, [C.c_char_p, _pd, C.POINTER(CheckpointHeader), _vp]),
    "nbgb_system_save": (C.c_int, [_vp, C.c_char_p, C.POINTER(CheckpointHeader), C.c_int32]),
    "nbgb_system_load": (C.c_int, [_vp, C.c_char_p, C.POINTER(_vp), C.POINTER(CheckpointHeader),
                                   _i32p]),
    "nbgb_measure_fp32_peak": (C.c_int, [_f64p, _f64p, _f64p]),
    "nbgb_direct_f64": (C.c_int, [_vp, C.c_int64, _vp, C.c_int64, C.c_double, C.c_double,
                                  _vp, _vp, _vp, _vp]),
    "nbgb_ensemble_config_default": (None, [C.POINTER(EnsembleConfig)]),
    "nbgb_ensemble_create": (C.c_int, [C.POINTER(EnsembleConfig), C.POINTER(_vp)]),
    "nbgb_ensemble_destroy": (C.c_int, [_vp]),
    "nbgb_ensemble_submit": (C.c_int, [_vp, _pd, C.c_int32, C.c_float, C.POINTER(C.c_uint64)]),
    "nbgb_ensemble_tick": (C.c_int, [_vp, _i32p, _i32p]),
    "nbgb_ensemble_poll": (C.c_int, [_vp, C.POINTER(EnsembleResult), _pd, _vp]),
    "nbgb_ensemble_synchronize": (C.c_int, [_vp]),
    "nbgb_ensemble_get_stats": (C.c_int, [_vp, C.POINTER(EnsembleStats)]),
    "nbgb_ensemble_get_stream": (C.c_int, [_vp, C.POINTER(_vp)]),
    "nbgb_last_error": (C.c_char_p, []),
    "nbgb_version": (C.c_char_p, []),
    "nbgb_abi_version": (C.c_int32, []),
}


def declared_symbols(header: str = _HEADER) -> list[str]:
    """Every function the public header declares (used by the ABI test)."""
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nbgb_[a-z0-9_]+)\s*\(", text)))


_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """Load (building first if needed) libnbgb.so and declare its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if not os.path.exists(path) or os.environ.get("NBGB_AUTOBUILD", "1") == "1":
        path = _build.build()
    handle = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(handle, name)
        fn.restype = res
        fn.argtypes = args
    _lib = handle
    return handle


def lib_path() -> str:
    return _build.LIB_PATH
