"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` may
import this module: it is the parity checker, never the thing measured.

``Oracle`` wraps ``liboracle.so`` (the C restatement of the reference path in
``nbody_oracle.c``).  ``Reference`` wraps ``_ref/libnbody_ref.so`` (the
reference's own host code, built in place from the reference sources) and is
only available where those sources exist.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build  # type: ignore[attr-defined]

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_i64 = C.c_int64
_f = C.c_float
_d = C.c_double

# OctreeNode, include/nbody/barnes_hut_tree.hpp:9-30 (76 bytes).
NODE_DTYPE = np.dtype([
    ("center", np.float32, 3), ("half", np.float32), ("com", np.float32, 3),
    ("mass", np.float32), ("children", np.int32, 8), ("particle_index", np.int32),
    ("is_leaf", np.uint8), ("pad", np.uint8, 3), ("particle_count", np.int32)])
assert NODE_DTYPE.itemsize == 76


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    """CPU restatement of the reference algorithm (see nbody_oracle.c)."""

    def __init__(self) -> None:
        lib = C.CDLL(_build.build_oracle())
        self.lib = lib
        lib.orc_pair_accel.argtypes = [_f32p, _f32p, _f, _f, _f, _f32p]
        lib.orc_direct_f32.argtypes = [_i64, _f32p, _f32p, _f32p, _f32p, _f, _f,
                                       _f32p, _f32p, _f32p, _i64, _i64]
        lib.orc_direct_f64.argtypes = [_i64, _f64p, _f64p, _f64p, _f64p, _d, _d,
                                       C.c_void_p, _i64, _f64p, _f64p, _f64p]
        lib.orc_update_positions.argtypes = [_i64] + [_f32p] * 9 + [_f]
        lib.orc_update_velocities.argtypes = [_i64] + [_f32p] * 9 + [_f]
        lib.orc_kinetic_energy.argtypes = [_i64, _f64p, _f64p, _f64p, _f64p]
        lib.orc_kinetic_energy.restype = _d
        lib.orc_potential_energy.argtypes = [_i64, _f64p, _f64p, _f64p, _f64p, _d, _d]
        lib.orc_potential_energy.restype = _d
        lib.orc_vv_step_f64.argtypes = [_i64] + [_f64p] * 10 + [_d, _d, _d]
        lib.orc_bbox.argtypes = [_i64, _f32p, _f32p, _f32p, _f32p, _f32p]
        lib.orc_morton_code.argtypes = [_f, _f, _f]
        lib.orc_morton_code.restype = C.c_uint32
        lib.orc_morton_keys.argtypes = [_i64, _f32p, _f32p, _f32p, _f32p, _f32p, _u32p, _i32p]
        lib.orc_stable_sort_u32.argtypes = [_i64, _u32p, _i32p]
        lib.orc_node_size.restype = C.c_int
        lib.orc_build_octree.argtypes = [_i64, _f32p, _f32p, _f32p, _f32p, _i32p, _f32p, _f32p,
                                         C.c_void_p, _i64, C.POINTER(C.c_int),
                                         C.POINTER(C.c_int), C.POINTER(C.c_int64)]
        lib.orc_bh_forces.argtypes = [C.c_void_p, C.c_int, _i64, _f32p, _f32p, _f32p, _f32p,
                                      _f, _f, _f, C.c_void_p, _i64, _f32p, _f32p, _f32p,
                                      C.c_void_p, C.c_int]
        lib.orc_bh_group_forces.argtypes = [C.c_void_p, C.c_int, _i64, _f32p, _f32p, _f32p,
                                            _f32p, _f, _f, _f, _f32p, _f32p, _f32p, C.c_void_p,
                                            C.c_int, C.c_int]
        lib.orc_hash_dims.argtypes = [_i64, _f32p, _f32p, _f32p, _f, _f32p, _f32p, _i32p,
                                      C.POINTER(C.c_int64)]
        lib.orc_cell_coords.argtypes = [_f, _f, _f, _f32p, _f, _i32p]
        lib.orc_hash_build.argtypes = [_i64, _f32p, _f32p, _f32p, _f, _f32p, _i32p, _i32p,
                                       _i32p, _i32p, _i32p]
        lib.orc_hash_forces.argtypes = [_i64, _f32p, _f32p, _f32p, _f32p, _f, _f32p, _i32p,
                                        _i32p, _i32p, _i32p, _f, _f, _f, C.c_void_p, _i64,
                                        _f32p, _f32p, _f32p, C.c_void_p]
        lib.orc_num_threads.restype = C.c_int
        lib.orc_set_num_threads.argtypes = [C.c_int]
        assert lib.orc_node_size() == 76

    # -- pair law / direct ---------------------------------------------------
    def pair_accel(self, p1, p2, m2, G, eps):
        out = np.zeros(3, np.float32)
        self.lib.orc_pair_accel(_f32(p1), _f32(p2), m2, G, eps, out)
        return out

    def direct_f32(self, x, y, z, m, G, eps, i_begin=0, i_end=None):
        x, y, z, m = map(_f32, (x, y, z, m))
        n = len(x)
        i_end = n if i_end is None else min(i_end, n)
        k = max(i_end - i_begin, 0)
        ax, ay, az = (np.zeros(k, np.float32) for _ in range(3))
        self.lib.orc_direct_f32(n, x, y, z, m, G, eps, ax, ay, az, i_begin, i_end)
        return ax, ay, az

    def direct_f64(self, x, y, z, m, G, eps, targets=None):
        x, y, z, m = map(_f64, (x, y, z, m))
        n = len(x)
        if targets is None:
            nt, tp = n, None
        else:
            t = np.ascontiguousarray(targets, dtype=np.int64)
            nt, tp = len(t), t.ctypes.data_as(C.c_void_p)
        ax, ay, az = (np.zeros(nt, np.float64) for _ in range(3))
        self.lib.orc_direct_f64(n, x, y, z, m, G, eps, tp, nt, ax, ay, az)
        return ax, ay, az

    # -- integrator ------------------------------------------------------------
    def update_positions(self, x, y, z, vx, vy, vz, ax, ay, az, dt):
        self.lib.orc_update_positions(len(x), x, y, z, vx, vy, vz, ax, ay, az, dt)

    def update_velocities(self, vx, vy, vz, aox, aoy, aoz, anx, any_, anz, dt):
        self.lib.orc_update_velocities(len(vx), vx, vy, vz, aox, aoy, aoz, anx, any_, anz, dt)

    def kinetic_energy(self, vx, vy, vz, m):
        vx, vy, vz, m = map(_f64, (vx, vy, vz, m))
        return self.lib.orc_kinetic_energy(len(vx), vx, vy, vz, m)

    def potential_energy(self, x, y, z, m, G, eps):
        x, y, z, m = map(_f64, (x, y, z, m))
        return self.lib.orc_potential_energy(len(x), x, y, z, m, G, eps)

    def vv_step_f64(self, s, m, G, eps, dt):
        """s: dict of float64 arrays x,y,z,vx,vy,vz,ax,ay,az (updated in place)."""
        self.lib.orc_vv_step_f64(len(m), s["x"], s["y"], s["z"], s["vx"], s["vy"], s["vz"],
                                 s["ax"], s["ay"], s["az"], _f64(m), G, eps, dt)

    # -- Barnes-Hut ------------------------------------------------------------
    def bbox(self, x, y, z):
        mn, mx = np.zeros(3, np.float32), np.zeros(3, np.float32)
        self.lib.orc_bbox(len(x), _f32(x), _f32(y), _f32(z), mn, mx)
        return mn, mx

    def morton_code(self, nx, ny, nz):
        return self.lib.orc_morton_code(nx, ny, nz)

    def morton_keys(self, x, y, z, bmin=None, bmax=None):
        x, y, z = map(_f32, (x, y, z))
        if bmin is None:
            bmin, bmax = self.bbox(x, y, z)
        n = len(x)
        keys = np.zeros(n, np.uint32)
        idx = np.zeros(n, np.int32)
        self.lib.orc_morton_keys(n, x, y, z, _f32(bmin), _f32(bmax), keys, idx)
        return keys, idx

    def stable_sort(self, keys, idx):
        k = np.array(keys, dtype=np.uint32, copy=True)
        v = np.array(idx, dtype=np.int32, copy=True)
        self.lib.orc_stable_sort_u32(len(k), k, v)
        return k, v

    def build_octree(self, x, y, z, m, sorted_idx, bmin, bmax, max_nodes=None):
        """Reference insertion octree; returns (nodes[:count], max_depth, budget_merges)."""
        x, y, z, m = map(_f32, (x, y, z, m))
        n = len(x)
        max_nodes = 2 * n if max_nodes is None else max_nodes
        nodes = np.zeros(max(max_nodes, 1), NODE_DTYPE)
        cnt, dep, merges = C.c_int(0), C.c_int(0), C.c_int64(0)
        rc = self.lib.orc_build_octree(n, x, y, z, m, np.ascontiguousarray(sorted_idx, np.int32),
                                       _f32(bmin), _f32(bmax), nodes.ctypes.data, max_nodes,
                                       C.byref(cnt), C.byref(dep), C.byref(merges))
        if rc != 0:
            raise OverflowError("oracle octree: node array overflow")
        return nodes[: cnt.value].copy(), dep.value, merges.value

    def bh_forces(self, nodes, x, y, z, m, theta, G, eps, targets=None, leaf_cap=1):
        x, y, z, m = map(_f32, (x, y, z, m))
        nodes = np.ascontiguousarray(nodes, NODE_DTYPE)
        n = len(x)
        if targets is None:
            nt, tp, tkeep = n, None, None
        else:
            tkeep = np.ascontiguousarray(targets, dtype=np.int64)
            nt, tp = len(tkeep), tkeep.ctypes.data_as(C.c_void_p)
        ax, ay, az = (np.zeros(nt, np.float32) for _ in range(3))
        inter = np.zeros(nt, np.int32)
        rc = self.lib.orc_bh_forces(nodes.ctypes.data, len(nodes), n, x, y, z, m, theta, G, eps,
                                    tp, nt, ax, ay, az, inter.ctypes.data, leaf_cap)
        if rc != 0:
            raise ValueError("oracle bucket walk: a bucket holds a multi-body leaf")
        return ax, ay, az, inter

    def bh_group_forces(self, nodes, x, y, z, m, theta, G, eps, leaf_capacity=1, group_max=32):
        """Group walk over the whole system: (ax, ay, az, interactions); with
        leaf_capacity > 1 opened buckets of at most that many bodies list them;
        group_max: the largest group (the library's choice for the body count)."""
        x, y, z, m = map(_f32, (x, y, z, m))
        nodes = np.ascontiguousarray(nodes, NODE_DTYPE)
        n = len(x)
        ax, ay, az = (np.zeros(n, np.float32) for _ in range(3))
        inter = np.zeros(n, np.int32)
        rc = self.lib.orc_bh_group_forces(nodes.ctypes.data, len(nodes), n, x, y, z, m, theta, G,
                                          eps, ax, ay, az, inter.ctypes.data, leaf_capacity,
                                          group_max)
        if rc != 0:
            raise ValueError("oracle group walk: multi-body leaves are not supported")
        return ax, ay, az, inter

    # -- spatial hash ------------------------------------------------------------
    def cell_coords(self, x, y, z, cell, bmin=(0.0, 0.0, 0.0)):
        """Unclamped cell coordinates floor((p - bmin) / cell) of one point."""
        out = np.zeros(3, np.int32)
        self.lib.orc_cell_coords(x, y, z, _f32(bmin), cell, out)
        return tuple(int(v) for v in out)

    def hash_dims(self, x, y, z, cell):
        """Padded box and grid dims of the hash grid; OverflowError above 1e8 cells."""
        x, y, z = map(_f32, (x, y, z))
        bmin, bmax = np.zeros(3, np.float32), np.zeros(3, np.float32)
        dims = np.zeros(3, np.int32)
        tot = C.c_int64(0)
        rc = self.lib.orc_hash_dims(len(x), x, y, z, cell, bmin, bmax, dims, C.byref(tot))
        if rc != 0:
            raise OverflowError("Spatial hash grid too large")
        return dict(bmin=bmin, bmax=bmax, dims=dims, total_cells=tot.value)

    def hash_build(self, x, y, z, cell):
        x, y, z = map(_f32, (x, y, z))
        n = len(x)
        bmin, bmax = np.zeros(3, np.float32), np.zeros(3, np.float32)
        dims = np.zeros(3, np.int32)
        tot = C.c_int64(0)
        rc = self.lib.orc_hash_dims(n, x, y, z, cell, bmin, bmax, dims, C.byref(tot))
        if rc != 0:
            raise OverflowError("Spatial hash grid too large")
        pc = np.zeros(n, np.int32)
        cs = np.zeros(tot.value, np.int32)
        ce = np.zeros(tot.value, np.int32)
        si = np.zeros(n, np.int32)
        self.lib.orc_hash_build(n, x, y, z, cell, bmin, dims, pc, cs, ce, si)
        return dict(bmin=bmin, bmax=bmax, dims=dims, particle_cell=pc, cell_start=cs,
                    cell_end=ce, sorted_indices=si, cell=np.float32(cell))

    def hash_forces(self, grid, x, y, z, m, cutoff, G, eps, targets=None):
        x, y, z, m = map(_f32, (x, y, z, m))
        n = len(x)
        if targets is None:
            nt, tp, tkeep = n, None, None
        else:
            tkeep = np.ascontiguousarray(targets, dtype=np.int64)
            nt, tp = len(tkeep), tkeep.ctypes.data_as(C.c_void_p)
        ax, ay, az = (np.zeros(nt, np.float32) for _ in range(3))
        nb = np.zeros(nt, np.int32)
        self.lib.orc_hash_forces(n, x, y, z, m, grid["cell"], grid["bmin"], grid["dims"],
                                 grid["cell_start"], grid["cell_end"], grid["sorted_indices"],
                                 cutoff, G, eps, tp, nt, ax, ay, az, nb.ctypes.data)
        return ax, ay, az, nb

    def num_threads(self) -> int:
        return self.lib.orc_num_threads()

    def set_num_threads(self, n: int) -> None:
        self.lib.orc_set_num_threads(n)


class Reference:
    """The reference's own host code (only where its sources exist)."""

    def __init__(self) -> None:
        path = _build.build_ref()
        if path is None:
            raise FileNotFoundError("reference sources not present")
        lib = C.CDLL(path)
        self.lib = lib
        lib.ref_pair_accel.argtypes = [_f32p, _f32p, _f, _f, _f, _f32p]
        lib.ref_morton_code.argtypes = [_f, _f, _f]
        lib.ref_morton_code.restype = C.c_uint32
        lib.ref_cell_index.argtypes = [_f, _f, _f, _f, _i32p]
        lib.ref_hash_grid_setup.argtypes = [_i64, _f32p, _f32p, _f32p, _f, _f32p, _f32p, _i32p,
                                            C.POINTER(C.c_int64)]
        lib.ref_init_spherical.argtypes = [_i64, _f, _f, _f, _f, _f, _f, C.c_uint] + [_f32p] * 7
        lib.ref_init_uniform.argtypes = [_i64, _f32p, _f32p, _f, _f, C.c_uint] + [_f32p] * 7
        lib.ref_build_tree.argtypes = [_i64, _f32p, _f32p, _f32p, _f32p, _i32p, _f32p, _f32p,
                                       C.c_void_p, _i64, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.ref_save_checkpoint.argtypes = [C.c_char_p, _i64, _f, _f, _f, _f, C.c_uint32] + \
            [_f32p] * 7
        lib.ref_load_checkpoint.argtypes = [C.c_char_p, C.POINTER(C.c_int64)] + \
            [C.POINTER(C.c_float)] * 4 + [C.POINTER(C.c_uint32)] + [C.c_void_p] * 7 + \
            [C.c_char_p, C.c_int]

    def pair_accel(self, p1, p2, m2, G, eps):
        out = np.zeros(3, np.float32)
        self.lib.ref_pair_accel(_f32(p1), _f32(p2), m2, G, eps, out)
        return out

    def morton_code(self, nx, ny, nz):
        return self.lib.ref_morton_code(nx, ny, nz)

    def cell_index(self, x, y, z, cell):
        out = np.zeros(3, np.int32)
        self.lib.ref_cell_index(x, y, z, cell, out)
        return tuple(int(v) for v in out)

    def hash_grid_setup(self, x, y, z, cell):
        """The reference's padded box and grid dims (SpatialHashGrid::build up to
        its first cell kernel); raises OverflowError where it rejects the grid."""
        x, y, z = map(_f32, (x, y, z))
        bmin, bmax = np.zeros(3, np.float32), np.zeros(3, np.float32)
        dims = np.zeros(3, np.int32)
        tot = C.c_int64(0)
        rc = self.lib.ref_hash_grid_setup(len(x), x, y, z, cell, bmin, bmax, dims, C.byref(tot))
        if rc == 2:
            raise OverflowError("Spatial hash grid too large")
        if rc != 0:
            raise RuntimeError("reference grid setup did not stop at its first cell kernel")
        return dict(bmin=bmin, bmax=bmax, dims=dims, total_cells=tot.value)

    def init_spherical(self, n, center=(0.0, 0.0, 0.0), radius=10.0, min_mass=1.0,
                       max_mass=1.0, seed=42):
        arrs = [np.zeros(n, np.float32) for _ in range(7)]
        self.lib.ref_init_spherical(n, *center, radius, min_mass, max_mass, seed, *arrs)
        return dict(zip(("x", "y", "z", "vx", "vy", "vz", "m"), arrs))

    def init_uniform(self, n, bmin, bmax, min_mass=1.0, max_mass=1.0, seed=42):
        arrs = [np.zeros(n, np.float32) for _ in range(7)]
        self.lib.ref_init_uniform(n, _f32(bmin), _f32(bmax), min_mass, max_mass, seed, *arrs)
        return dict(zip(("x", "y", "z", "vx", "vy", "vz", "m"), arrs))

    def build_tree(self, x, y, z, m, sorted_idx, bmin, bmax):
        x, y, z, m = map(_f32, (x, y, z, m))
        n = len(x)
        nodes = np.zeros(max(2 * n, 1), NODE_DTYPE)
        cnt, dep = C.c_int(0), C.c_int(0)
        rc = self.lib.ref_build_tree(n, x, y, z, m, np.ascontiguousarray(sorted_idx, np.int32),
                                     _f32(bmin), _f32(bmax), nodes.ctypes.data, len(nodes),
                                     C.byref(cnt), C.byref(dep))
        if rc != 0:
            raise OverflowError("reference tree larger than its node array")
        return nodes[: cnt.value].copy(), dep.value

    def save_checkpoint(self, path, s, sim_time=0.0, dt=1e-3, G=1.0, softening=0.1, method=0):
        arrs = [_f32(s[k]) for k in ("x", "y", "z", "vx", "vy", "vz", "m")]
        rc = self.lib.ref_save_checkpoint(os.fsencode(path), len(arrs[0]), sim_time, dt, G,
                                          softening, method, *arrs)
        if rc != 0:
            raise IOError("reference save failed")

    def load_checkpoint(self, path):
        """Returns (header dict, arrays dict) or raises ValueError with the reference's text."""
        n = C.c_int64(0)
        st, dt, G, eps = C.c_float(0), C.c_float(0), C.c_float(0), C.c_float(0)
        meth = C.c_uint32(0)
        err = C.create_string_buffer(512)
        nulls = [None] * 7
        rc = self.lib.ref_load_checkpoint(os.fsencode(path), C.byref(n), C.byref(st), C.byref(dt),
                                          C.byref(G), C.byref(eps), C.byref(meth), *nulls, err,
                                          512)
        if rc != 0:
            raise ValueError(err.value.decode())
        arrs = [np.zeros(n.value, np.float32) for _ in range(7)]
        rc = self.lib.ref_load_checkpoint(os.fsencode(path), C.byref(n), C.byref(st), C.byref(dt),
                                          C.byref(G), C.byref(eps), C.byref(meth),
                                          *[a.ctypes.data for a in arrs], err, 512)
        hdr = dict(particle_count=n.value, simulation_time=st.value, dt=dt.value, G=G.value,
                   softening=eps.value, force_method=meth.value)
        return hdr, dict(zip(("x", "y", "z", "vx", "vy", "vz", "m"), arrs))
