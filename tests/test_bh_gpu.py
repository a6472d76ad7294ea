"""Barnes-Hut through the C ABI vs the oracle and the reference (GPU).

Bit-exact: Morton keys and the stably sorted (key, index) pairs; the octree
(topology and every node's mass, centre of mass, centre, half size, leaf
body, body count) against the reference's host insertion build -- golden
node arrays produced by the reference's own code, and the oracle's
restatement of it (pinned bit-exact to those goldens) for larger inputs;
per-target accepted-interaction counts against the oracle walk (one body
per leaf, and the bucket walk over subtrees of at most 2..16 bodies).
Forces within 1e-5 (p99, vector relative) of the oracle walk on the same
tree; theta = 0.5 with 8-body buckets median relative error <= 2e-3 against
the FP64 direct sum.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err, vec_rel_err
from treeutil import compare

pytestmark = pytest.mark.gpu


def _bh(nb, s, theta=0.5, eps=0.01, leaf=1, count=True, G=1.0, group=False, ref_tree=False):
    calc = nb.BarnesHutCalculator(theta, leaf_capacity=leaf, group_walk=group)
    calc.setGravitationalConstant(G)
    calc.setSofteningParameter(eps)
    if count or ref_tree:
        calc.set_flags(nb.FLAG_SYNC | nb.FLAG_COMPENSATED |
                       (nb.FLAG_COUNT_INTERACTIONS if count else 0) |
                       (nb.FLAG_GROUP_WALK if group else 0) |
                       (nb.FLAG_REFERENCE_TREE if ref_tree else 0))
    n = len(s["x"])
    with nb.ScopedParticleData(n, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                   "mass": s["m"]}) as p:
        calc.computeForces(p.device)
        p.download()
        acc = (p.host["acc_x"].copy(), p.host["acc_y"].copy(), p.host["acc_z"].copy())
    out = dict(acc=acc, keys=calc.sorted_keys(n), nodes=calc.nodes(), stats=calc.tree_stats())
    if count:
        out["inter"] = calc.interaction_counts(n)
    calc.close()
    return out


def _gmax(nb, s):
    """The largest group the library forms for this many bodies (32 or 64)."""
    return int(nb.lib().nbgb_bh_group_size(len(s["x"])))


def _oracle_tree(orc, s, max_nodes=None):
    bmin, bmax = orc.bbox(s["x"], s["y"], s["z"])
    keys, idx = orc.morton_keys(s["x"], s["y"], s["z"], bmin, bmax)
    ks, si = orc.stable_sort(keys, idx)
    nodes, depth, merges = orc.build_octree(s["x"], s["y"], s["z"], s["m"], si, bmin, bmax,
                                            max_nodes=max_nodes)
    return ks, si, nodes, depth, merges


def _golden_tree(golden, name):
    from oracle.oracle import NODE_DTYPE
    g = golden("ref_trees.npz")
    s = {k: g[f"{name}_{k}"] for k in ("x", "y", "z", "m")}
    nodes = np.frombuffer(g[f"{name}_nodes"].tobytes(), NODE_DTYPE)
    return s, g[f"{name}_keys"], g[f"{name}_sorted"], nodes, int(g[f"{name}_depth"])


@pytest.mark.parametrize("name", ["sph100", "sph700", "uni500"])
def test_tree_matches_reference_golden(nb, golden, name):
    s, keys, order, ref_nodes, ref_depth = _golden_tree(golden, name)
    r = _bh(nb, s)
    np.testing.assert_array_equal(r["keys"][0], keys)
    np.testing.assert_array_equal(r["keys"][1], order)
    assert compare(r["nodes"], ref_nodes) == []
    assert r["stats"] == (len(ref_nodes), ref_depth)


@pytest.mark.parametrize("gen,n", [("plummer", 5000), ("plummer", 65536), ("two", 100000),
                                   ("cube", 30000)])
def test_tree_matches_reference_insertion(nb, orc, gen, n):
    s = {"plummer": lambda: nb.ics.plummer(n, seed=n), "two": lambda: nb.ics.two_plummer(n, seed=2),
         "cube": lambda: nb.ics.uniform_cube(n, seed=4)}[gen]()
    ks, si, nodes, depth, merges = _oracle_tree(orc, s)
    assert merges == 0  # the reference's 2N budget does not fire at these sizes
    r = _bh(nb, s)
    np.testing.assert_array_equal(r["keys"][0], ks)
    np.testing.assert_array_equal(r["keys"][1], si)
    assert compare(r["nodes"], nodes) == []
    assert r["stats"] == (len(nodes), depth)


@pytest.mark.parametrize("name", ["sph30", "sph100", "sph700", "uni500", "coincident16",
                                  "collinear16"])
def test_reference_tree_mode_matches_reference_golden(nb, golden, name):
    """NBGB_FLAG_REFERENCE_TREE: node for node the tree the reference's own
    host build made, including the cases where its 2N node budget merges
    bodies into multi-body leaves (sph30: 9 bodies) and the degenerate
    coincident / collinear inputs."""
    s, keys, order, ref_nodes, ref_depth = _golden_tree(golden, name)
    r = _bh(nb, s, ref_tree=True)
    np.testing.assert_array_equal(r["keys"][1], order)
    assert compare(r["nodes"], ref_nodes) == []
    assert r["stats"] == (len(ref_nodes), ref_depth)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 30, 50, 64, 100, 300, 2000])
def test_reference_tree_mode_matches_oracle_budget_tree_and_walk(nb, orc, n):
    """The reference-identical tree against the oracle's restatement of the
    reference build (2N budget), and the reference walk on it: interaction
    counts bit-exact, forces within 1e-5 (p99) of the oracle walk."""
    s = nb.ics.plummer(n, seed=40 + n)
    _, _, nodes, depth, merges = _oracle_tree(orc, s)
    r = _bh(nb, s, ref_tree=True)
    assert compare(r["nodes"], nodes) == []
    assert r["stats"] == (len(nodes), depth)
    ox, oy, oz, oint = orc.bh_forces(nodes, s["x"], s["y"], s["z"], s["m"], 0.5, 1.0, 0.01)
    np.testing.assert_array_equal(r["inter"], oint)
    has = np.abs(ox) + np.abs(oy) + np.abs(oz) > 0
    if has.any():
        err = vec_rel_err(*(a[has] for a in r["acc"]), ox[has], oy[has], oz[has])
        assert np.percentile(err, 99) <= 1e-5, np.percentile(err, 99)


def test_reference_tree_mode_merges_where_the_budget_fires(nb, orc):
    # the budget fires for some of these small systems, and the default
    # (canonical) build then differs from the reference-identical one
    fired = 0
    for n in (20, 30, 40, 50):
        s = nb.ics.plummer(n, seed=40 + n)
        _, _, nodes, _, merges = _oracle_tree(orc, s)
        if merges:
            fired += 1
            assert compare(_bh(nb, s)["nodes"], nodes) != []
            assert compare(_bh(nb, s, ref_tree=True)["nodes"], nodes) == []
    assert fired > 0


@pytest.mark.parametrize("n", [30, 2000])
def test_reference_tree_mode_asynchronous(nb, orc, n):
    # without NBGB_FLAG_SYNC the reference's insertion is always replayed
    s = nb.ics.plummer(n, seed=40 + n)
    _, _, nodes, depth, _ = _oracle_tree(orc, s)
    calc = nb.BarnesHutCalculator(0.5)
    calc.setSofteningParameter(0.01)
    calc.set_flags(nb.FLAG_COMPENSATED | nb.FLAG_REFERENCE_TREE)
    with nb.ScopedParticleData(n, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                   "mass": s["m"]}) as p:
        calc.computeForces(p.device)
        calc.synchronize()
        p.download()
    assert compare(calc.nodes(), nodes) == []
    assert calc.tree_stats() == (len(nodes), depth)
    ox, oy, oz, _ = orc.bh_forces(nodes, s["x"], s["y"], s["z"], s["m"], 0.5, 1.0, 0.01)
    err = vec_rel_err(p.host["acc_x"], p.host["acc_y"], p.host["acc_z"], ox, oy, oz)
    assert np.percentile(err, 99) <= 1e-5
    calc.close()


def test_reference_tree_mode_limits(nb):
    calc = nb.BarnesHutCalculator(0.5, group_walk=True)
    with pytest.raises(nb.ValidationException):
        calc.set_flags(nb.FLAG_SYNC | nb.FLAG_GROUP_WALK | nb.FLAG_REFERENCE_TREE)
    calc.close()
    big = nb.ics.plummer(65537, seed=4)
    arrays = {"pos_x": big["x"], "pos_y": big["y"], "pos_z": big["z"], "mass": big["m"]}
    # asynchronously the replay always runs, and is limited to 65,536 bodies
    calc = nb.BarnesHutCalculator(0.5)
    calc.set_flags(nb.FLAG_REFERENCE_TREE)
    with nb.ScopedParticleData(65537, arrays) as p:
        with pytest.raises(nb.ValidationException, match="65536"):
            calc.computeForces(p.device)
    calc.close()
    # synchronously it runs only where the trees can differ: not here
    calc = nb.BarnesHutCalculator(0.5)
    calc.set_flags(nb.FLAG_SYNC | nb.FLAG_REFERENCE_TREE)
    with nb.ScopedParticleData(65537, arrays) as p:
        calc.computeForces(p.device)
    calc.close()


def test_keys_with_duplicates_are_stable(nb, orc):
    rng = np.random.default_rng(1)
    base = rng.uniform(-1, 1, (40, 3)).astype(np.float32)
    pts = base[rng.integers(0, 40, 3000)]  # many identical positions -> equal keys
    s = dict(x=pts[:, 0].copy(), y=pts[:, 1].copy(), z=pts[:, 2].copy(),
             m=rng.uniform(0.5, 1.5, 3000).astype(np.float32))
    r = _bh(nb, s)
    ks, si, nodes, _, _ = _oracle_tree(orc, s, max_nodes=64 * 3000)
    np.testing.assert_array_equal(r["keys"][0], ks)
    np.testing.assert_array_equal(r["keys"][1], si)
    # depth-32 multi-body leaves: merged in Morton (insertion) order
    assert compare(r["nodes"], nodes) == []


@pytest.mark.parametrize("gen,n,theta", [("plummer", 4096, 0.5), ("plummer", 20000, 0.3),
                                         ("two", 50000, 0.5), ("plummer", 3000, 1.0),
                                         ("far", 6000, 0.5), ("dense", 6000, 0.5)])
def test_interaction_sets_and_forces_match_oracle_walk(nb, orc, gen, n, theta):
    """Interaction sets per target equal the oracle's (which tests cube
    containment at every node); 'far' is a cluster 2000 units from the
    origin (coordinate rounding comparable to the cells), 'dense' a cluster
    whose cells shrink below the softening length."""
    if gen == "plummer":
        s = nb.ics.plummer(n, seed=n)
    elif gen == "two":
        s = nb.ics.two_plummer(n, seed=3)
    elif gen == "far":
        s = nb.ics.plummer(n, seed=11, center=(2000.0, -1500.0, 700.0))
    else:
        s = nb.ics.plummer(n, seed=12, a=0.01)
    _, _, nodes, _, merges = _oracle_tree(orc, s)
    assert merges == 0
    r = _bh(nb, s, theta=theta)
    t = np.random.default_rng(5).choice(n, min(n, 4096), replace=False)
    ox, oy, oz, oint = orc.bh_forces(nodes, s["x"], s["y"], s["z"], s["m"], theta, 1.0, 0.01,
                                     targets=t)
    np.testing.assert_array_equal(r["inter"][t], oint)
    ax, ay, az = (a[t] for a in r["acc"])
    err = vec_rel_err(ax, ay, az, ox, oy, oz)
    assert np.percentile(err, 99) <= 1e-5, np.percentile(err, 99)


@pytest.mark.parametrize("gen,n,theta,leaf", [("plummer", 20000, 0.5, 8), ("two", 50000, 0.5, 8),
                                              ("plummer", 6000, 0.3, 2), ("plummer", 6000, 0.8, 16),
                                              ("dense", 6000, 0.5, 8)])
def test_bucket_interaction_sets_match_oracle_walk(nb, orc, gen, n, theta, leaf):
    """Bucket walk (subtrees of at most `leaf` bodies summed directly):
    per-target interaction counts equal the oracle's bucket walk on the same
    tree, forces within 1e-5 (p99, vector relative)."""
    if gen == "plummer":
        s = nb.ics.plummer(n, seed=n + leaf)
    elif gen == "two":
        s = nb.ics.two_plummer(n, seed=4)
    else:
        s = nb.ics.plummer(n, seed=13, a=0.01)
    _, _, nodes, _, merges = _oracle_tree(orc, s)
    assert merges == 0
    r = _bh(nb, s, theta=theta, leaf=leaf)
    t = np.random.default_rng(6).choice(n, min(n, 4096), replace=False)
    ox, oy, oz, oint = orc.bh_forces(nodes, s["x"], s["y"], s["z"], s["m"], theta, 1.0, 0.01,
                                     targets=t, leaf_cap=leaf)
    np.testing.assert_array_equal(r["inter"][t], oint)
    err = vec_rel_err(*(a[t] for a in r["acc"]), ox, oy, oz)
    assert np.percentile(err, 99) <= 1e-5, np.percentile(err, 99)


def _gen(nb, gen, n):
    return {"plummer": lambda: nb.ics.plummer(n, seed=n),
            "two": lambda: nb.ics.two_plummer(n, seed=3),
            "cube": lambda: nb.ics.uniform_cube(n, seed=4),
            "far": lambda: nb.ics.plummer(n, seed=11, center=(2000.0, -1500.0, 700.0)),
            "dense": lambda: nb.ics.plummer(n, seed=12, a=0.01)}[gen]()


@pytest.mark.parametrize("gen,n,theta,eps", [("plummer", 5000, 0.5, 0.01), ("plummer", 20000, 0.3, 0.01),
                                             ("two", 50000, 0.5, 0.01), ("cube", 30000, 0.5, 0.01),
                                             ("far", 6000, 0.5, 0.01), ("dense", 6000, 0.5, 0.01),
                                             ("plummer", 3000, 1.0, 0.01), ("plummer", 4000, 0.5, 0.0),
                                             ("plummer", 3000, 2.0, 0.01), ("cube", 5000, 0.5, 5.0),
                                             ("two", 300000, 0.5, 0.01), ("plummer", 262144, 0.5, 0.0)])
def test_group_walk_matches_oracle(nb, orc, gen, n, theta, eps):
    """Group walk: per-body list lengths (interactions) equal the oracle's
    group walk on the same tree -- same groups, same bounding boxes, same
    acceptance arithmetic -- and forces agree within 1e-5 (p99, vector
    relative; the list order differs).  eps = 0 runs the zero-softening
    variant (zero-distance entries add nothing).  From 262,144 bodies on the
    groups hold up to 64 bodies, two per lane."""
    s = _gen(nb, gen, n)
    _, _, nodes, _, merges = _oracle_tree(orc, s)
    assert merges == 0
    r = _bh(nb, s, theta=theta, eps=eps, group=True)
    ox, oy, oz, oint = orc.bh_group_forces(nodes, s["x"], s["y"], s["z"], s["m"], theta, 1.0, eps,
                                           group_max=_gmax(nb, s))
    np.testing.assert_array_equal(r["inter"], oint)
    err = vec_rel_err(*r["acc"], ox, oy, oz)
    assert np.percentile(err, 99) <= 1e-5, np.percentile(err, 99)


def test_group_walk_theta0_is_direct_sum(nb, orc):
    n = 3000
    s = nb.ics.plummer(n, seed=21)
    r = _bh(nb, s, theta=0.0, group=True)
    assert (r["inter"] == n - 1).all()
    bx, by, bz = orc.direct_f64(s["x"], s["y"], s["z"], s["m"], 1.0, 0.01)
    assert np.max(vec_rel_err(*r["acc"], bx, by, bz)) < 1e-4


@pytest.mark.parametrize("gen,n,leaf", [("two", 300000, 1), ("plummer", 20000, 1), ("two", 50000, 8)])
def test_group_order_does_not_change_results(nb, gen, n, leaf):
    """The walk takes the groups in cost classes learned from the previous
    evaluation (the first evaluation has none): repeated evaluations of the
    same bodies give bitwise-identical accelerations and list lengths."""
    s = _gen(nb, gen, n)
    calc = nb.BarnesHutCalculator(0.5, leaf_capacity=leaf, group_walk=True)
    calc.setSofteningParameter(0.01)
    calc.set_flags(nb.FLAG_SYNC | nb.FLAG_COMPENSATED | nb.FLAG_COUNT_INTERACTIONS |
                   nb.FLAG_GROUP_WALK)
    runs = []
    with nb.ScopedParticleData(n, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                   "mass": s["m"]}) as p:
        for _ in range(3):
            calc.computeForces(p.device)
            p.download()
            runs.append((p.host["acc_x"].copy(), p.host["acc_y"].copy(), p.host["acc_z"].copy(),
                         calc.interaction_counts(n)))
    calc.close()
    for r in runs[1:]:
        for a, b in zip(runs[0], r):
            np.testing.assert_array_equal(a, b)


def test_group_walk_is_more_accurate_than_reference_walk(nb, orc):
    # every accepted cell passes the per-target test for each body of the group
    n = 65536
    s = nb.ics.two_plummer(n, seed=8)
    t = np.random.default_rng(9).choice(n, 2048, replace=False)
    bx, by, bz = orc.direct_f64(s["x"], s["y"], s["z"], s["m"], 1.0, 0.01, targets=t)
    e1 = vec_rel_err(*(a[t] for a in _bh(nb, s, count=False)["acc"]), bx, by, bz)
    eg = vec_rel_err(*(a[t] for a in _bh(nb, s, count=False, group=True)["acc"]), bx, by, bz)
    assert np.median(eg) < np.median(e1) and np.median(eg) <= 1e-3, (np.median(eg), np.median(e1))


@pytest.fixture
def small_group_stack(nb):
    from nbgb import _lib
    nb.check(_lib.lib().nbgb_selftest_group_walk_stack(64))
    yield
    nb.check(_lib.lib().nbgb_selftest_group_walk_stack(512))


def test_group_walk_spill_path(nb, orc, small_group_stack):
    """With a 64-entry shared stack every group spills to its global overflow
    chunk and reloads: the same lists as the oracle's."""
    n = 1500
    s = nb.ics.plummer(n, seed=22)
    _, _, nodes, _, _ = _oracle_tree(orc, s)
    r = _bh(nb, s, theta=0.2, group=True)
    ox, oy, oz, oint = orc.bh_group_forces(nodes, s["x"], s["y"], s["z"], s["m"], 0.2, 1.0, 0.01,
                                           group_max=_gmax(nb, s))
    np.testing.assert_array_equal(r["inter"], oint)
    assert np.percentile(vec_rel_err(*r["acc"], ox, oy, oz), 99) <= 1e-5


def test_group_walk_overflow_is_reported(nb, small_group_stack):
    """More spilling warps than overflow chunks: the walk reports an overflow
    status (no fault), and the next call with the normal stack succeeds."""
    from nbgb import _lib
    n = 20000
    s = nb.ics.plummer(n, seed=23)
    with pytest.raises(nb.NbodyError, match="group walk stack overflow"):
        _bh(nb, s, theta=0.0, group=True)
    nb.check(_lib.lib().nbgb_selftest_group_walk_stack(512))
    r = _bh(nb, s, theta=0.5, group=True)
    assert np.isfinite(r["acc"][0]).all()


@pytest.mark.parametrize("gen,n,theta,leaf", [("plummer", 5000, 0.5, 8), ("two", 50000, 0.5, 8),
                                              ("cube", 30000, 0.5, 4), ("dense", 6000, 0.5, 16),
                                              ("plummer", 3000, 1.0, 2), ("far", 6000, 0.3, 8)])
def test_group_walk_buckets_match_oracle(nb, orc, gen, n, theta, leaf):
    """Group walk over buckets (an opened node of at most `leaf` bodies lists
    its bodies): per-body list lengths equal the oracle's bucket group walk on
    the same tree, forces within 1e-5 of it (p99, vector relative)."""
    s = _gen(nb, gen, n)
    _, _, nodes, _, merges = _oracle_tree(orc, s)
    assert merges == 0
    r = _bh(nb, s, theta=theta, leaf=leaf, group=True)
    ox, oy, oz, oint = orc.bh_group_forces(nodes, s["x"], s["y"], s["z"], s["m"], theta, 1.0,
                                           0.01, leaf, group_max=_gmax(nb, s))
    np.testing.assert_array_equal(r["inter"], oint)
    err = vec_rel_err(*r["acc"], ox, oy, oz)
    assert np.percentile(err, 99) <= 1e-5, np.percentile(err, 99)


def test_group_walk_buckets_with_coincident_bodies(nb, orc):
    # small depth-32 leaves inside buckets and a large one (listed 32 at a time)
    n = 4000
    s = nb.ics.plummer(n, seed=31)
    for k in ("x", "y", "z"):
        s[k][100:105] = s[k][100]   # a 5-body depth-32 leaf
        s[k][200:300] = s[k][200]   # a 100-body depth-32 leaf
    bx, by, bz = orc.direct_f64(s["x"], s["y"], s["z"], s["m"], 1.0, 0.01)
    for leaf in (1, 8):
        r = _bh(nb, s, theta=0.0, leaf=leaf, group=True)
        assert (r["inter"] == n - 1).all()
        assert np.max(vec_rel_err(*r["acc"], bx, by, bz)) < 1e-4


def test_small_theta_matches_direct(nb, golden):
    # tests/test_spatial_hash.cpp:171-228: theta = 0.1 vs direct < 2 % per
    # component (the canonical tree; the reference's 2N budget merge would
    # fail this bound at N = 30, see test_oracle_pins)
    g = golden("ref_inputs.npz")
    s = {k: g[f"sph30_r5_{k}"] for k in ("x", "y", "z", "m")}
    r = _bh(nb, s, theta=0.1, eps=0.1)
    calc = nb.DirectForceCalculator()
    calc.setSofteningParameter(0.1)
    with nb.ScopedParticleData(30, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                    "mass": s["m"]}) as p:
        calc.computeForces(p.device)
        p.download()
        d = (p.host["acc_x"], p.host["acc_y"], p.host["acc_z"])
    calc.close()
    err = max(rel_err(a, b, 1e-4).max() for a, b in zip(r["acc"], d))
    assert err < 0.02


def test_theta_convergence(nb, orc, golden):
    # tests/test_barnes_hut.cpp:168-220
    g = golden("ref_inputs.npz")
    s = {k: g[f"sph50_r10_{k}"] for k in ("x", "y", "z", "m")}
    dx, dy, dz = orc.direct_f32(s["x"], s["y"], s["z"], s["m"], 1.0, 0.1)

    def total(theta):
        ax, ay, az = _bh(nb, s, theta=theta, eps=0.1)["acc"]
        return np.sum(np.sqrt((ax - dx) ** 2 + (ay - dy) ** 2 + (az - dz) ** 2))

    assert total(0.3) <= 1.1 * total(0.8)


def test_degenerate_sets_conserve_mass_and_stay_finite(nb):
    # tests/test_barnes_hut.cpp:53-89,116-138
    n = 16
    same = dict(x=np.full(n, 1.0, np.float32), y=np.full(n, 2.0, np.float32),
                z=np.full(n, 3.0, np.float32), m=np.ones(n, np.float32))
    line = dict(x=(np.float32(1e-4) * np.arange(n, dtype=np.float32)).astype(np.float32),
                y=np.zeros(n, np.float32), z=np.zeros(n, np.float32), m=np.ones(n, np.float32))
    for s in (same, line):
        r = _bh(nb, s, eps=0.1)
        assert abs(r["nodes"][0]["mass"] - n) < 1e-3 * n
        assert all(np.all(np.isfinite(a)) for a in r["acc"])
    r = _bh(nb, same, eps=0.1)
    assert r["stats"][1] == 32  # all bodies in one depth-32 leaf
    # self-subtraction leaves the other 15 bodies at the target's own position
    assert all(np.all(np.abs(a) < 1e-3) for a in r["acc"])


@pytest.mark.parametrize("n", [1, 2, 3, 31, 33])
def test_tiny_systems(nb, orc, n):
    s = nb.ics.plummer(n, seed=40 + n)
    r = _bh(nb, s, theta=0.0)
    if n == 1:
        assert all(a[0] == 0.0 for a in r["acc"])
        assert r["stats"] == (2, 0)
        return
    bx, by, bz = orc.direct_f64(s["x"], s["y"], s["z"], s["m"], 1.0, 0.01)
    assert np.max(vec_rel_err(*r["acc"], bx, by, bz)) < 1e-4  # theta = 0: exact up to rounding


def test_bucket_leaves_accuracy(nb, orc):
    n = 65536
    s = nb.ics.two_plummer(n, seed=8)
    t = np.random.default_rng(9).choice(n, 2048, replace=False)
    bx, by, bz = orc.direct_f64(s["x"], s["y"], s["z"], s["m"], 1.0, 0.01, targets=t)
    for leaf in (1, 8):
        ax, ay, az = (a[t] for a in _bh(nb, s, theta=0.5, leaf=leaf, count=False)["acc"])
        err = vec_rel_err(ax, ay, az, bx, by, bz)
        assert np.median(err) <= 2e-3, (leaf, np.median(err))


@pytest.mark.slow
def test_full_size_two_plummer(nb, orc):
    # The Barnes-Hut workload: N = 1,048,576 two Plummer spheres, theta = 0.5,
    # eps = 0.01.  Keys, order and tree bit-exact against the reference
    # insertion build; forces on 4096 seeded targets vs the FP64 direct sum.
    n = 1 << 20
    s = nb.ics.two_plummer(n, seed=2)
    ks, si, nodes, depth, merges = _oracle_tree(orc, s)
    assert merges == 0
    r = _bh(nb, s, theta=0.5, leaf=1, count=False)
    np.testing.assert_array_equal(r["keys"][0], ks)
    np.testing.assert_array_equal(r["keys"][1], si)
    assert r["stats"] == (len(nodes), depth)
    assert compare(r["nodes"], nodes) == []
    t = np.random.default_rng(2).choice(n, 4096, replace=False)
    bx, by, bz = orc.direct_f64(s["x"], s["y"], s["z"], s["m"], 1.0, 0.01, targets=t)
    err = vec_rel_err(*(a[t] for a in r["acc"]), bx, by, bz)
    assert np.median(err) <= 2e-3
    # the same workload with 8-body buckets: interaction sets equal the
    # oracle's bucket walk on the same tree, and the same error bound
    r8 = _bh(nb, s, theta=0.5, leaf=8)
    _, _, _, oint = orc.bh_forces(nodes, s["x"], s["y"], s["z"], s["m"], 0.5, 1.0, 0.01,
                                  targets=t, leaf_cap=8)
    np.testing.assert_array_equal(r8["inter"][t], oint)
    err8 = vec_rel_err(*(a[t] for a in r8["acc"]), bx, by, bz)
    assert np.median(err8) <= 2e-3
    # and with the group walk: every body's list length equals the oracle's
    # group walk on the same tree, forces within 1e-5 of it, and a lower
    # error against FP64 than the reference walk
    rg = _bh(nb, s, theta=0.5, group=True)
    assert _gmax(nb, s) == 64  # a build this large forms groups of up to 64 bodies
    ox, oy, oz, oint = orc.bh_group_forces(nodes, s["x"], s["y"], s["z"], s["m"], 0.5, 1.0, 0.01,
                                           group_max=64)
    np.testing.assert_array_equal(rg["inter"], oint)
    assert np.percentile(vec_rel_err(*rg["acc"], ox, oy, oz), 99) <= 1e-5
    errg = vec_rel_err(*(a[t] for a in rg["acc"]), bx, by, bz)
    assert np.median(errg) <= np.median(err)
    # the workload as configured (leaf <= 8 bodies) on the group walk: list
    # lengths equal the oracle's bucket group walk, forces within 1e-5 of it,
    # median error <= 2e-3 and no worse than either reference-style walk
    rg8 = _bh(nb, s, theta=0.5, leaf=8, group=True)
    ox, oy, oz, oint = orc.bh_group_forces(nodes, s["x"], s["y"], s["z"], s["m"], 0.5, 1.0, 0.01,
                                           8, group_max=64)
    np.testing.assert_array_equal(rg8["inter"], oint)
    assert np.percentile(vec_rel_err(*rg8["acc"], ox, oy, oz), 99) <= 1e-5
    errg8 = vec_rel_err(*(a[t] for a in rg8["acc"]), bx, by, bz)
    assert np.median(errg8) <= 2e-3
    assert np.median(errg8) <= min(np.median(err), np.median(err8))

