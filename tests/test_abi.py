"""The C-ABI library builds for sm_103a, loads, and exports every symbol the
public header declares.  CPU only: no compute call is made."""
from __future__ import annotations

import ctypes as C
import subprocess

import pytest


def test_library_exports_every_declared_symbol(nb):
    lib = nb.lib()
    declared = nb.declared_symbols()
    assert len(declared) >= 30
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", nb.lib_path()], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(declared) <= exported


def test_library_is_sm103a_only(nb):
    out = subprocess.run(["cuobjdump", "--list-elf", nb.lib_path()], capture_output=True,
                         text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    arches = {tok for tok in out.stdout.split() if "sm_" in tok}
    assert arches and all("sm_103a" in a for a in arches), arches


def test_abi_version_and_defaults(nb):
    lib = nb.lib()
    assert lib.nbgb_abi_version() == 2
    assert b"sm_103a" in lib.nbgb_version()
    p = nb.default_params()
    # SimulationConfig defaults (include/nbody/types.hpp:133-144)
    assert (p.G, p.softening, p.theta, p.cell_size, p.cutoff, p.block_size) == \
        (1.0, pytest.approx(0.1), 0.5, 2.0, 2.0, 256)
    assert p.leaf_capacity == 1 and p.group_size == 0
    assert p.flags & nb.FLAG_SYNC and p.flags & nb.FLAG_COMPENSATED
    # the drop-in calculator walks the tree as the reference does; the
    # serving engine defaults to the group walk
    assert not p.flags & nb.FLAG_GROUP_WALK
    assert nb.BarnesHutCalculator.__init__.__defaults__[-2] is False  # group_walk
    from nbgb.serving import default_config
    cfg = default_config()
    assert cfg.group_walk == 1 and cfg.leaf_capacity == 1 and cfg.theta == 0.5


def test_struct_layouts_match_reference(nb):
    from nbgb._lib import ParticleDataStruct, OctreeNode
    assert C.sizeof(ParticleDataStruct) == 112
    assert ParticleDataStruct.mass.offset == 96 and ParticleDataStruct.count.offset == 104
    assert C.sizeof(OctreeNode) == 76
    assert OctreeNode.half_size.offset == 12 and OctreeNode.center_of_mass.offset == 16
    assert OctreeNode.total_mass.offset == 28 and OctreeNode.children.offset == 32
    assert OctreeNode.particle_index.offset == 64 and OctreeNode.is_leaf.offset == 68
    assert OctreeNode.particle_count.offset == 72


def test_method_enum_matches_reference(nb):
    assert [int(m) for m in nb.ForceMethod] == [0, 1, 2]
    assert nb.forceMethodToString(nb.ForceMethod.BARNES_HUT) == "barnes_hut"


def test_group_walk_stack_hook_validates(nb):
    # process-wide test hook of the group walk; no device work
    lib = nb.lib()
    assert lib.nbgb_selftest_group_walk_stack(63) == 1  # NBGB_ERR_INVALID_ARG
    assert lib.nbgb_selftest_group_walk_stack(513) == 1
    assert lib.nbgb_selftest_group_walk_stack(512) == 0  # the default


def test_group_size_rule(nb):
    """The group walk's largest group: 32 bodies below 262,144 bodies per
    build, 64 from there on (host-only call)."""
    f = nb.lib().nbgb_bh_group_size
    assert [f(n) for n in (0, 1, 1000, 262143)] == [32] * 4
    assert [f(n) for n in (262144, 1 << 20, 1 << 40)] == [64] * 3
