"""Spatial hash through the C ABI vs the oracle (GPU).

Bit-exact: grid dims, padded bbox, cell_start/cell_end, per-particle cell
ids, the cell-ordered index list (ascending index within a cell, the order
the oracle fixes) and per-target neighbour counts.  Forces: per target
|a - a_oracle| / |a_oracle| <= 1e-5 at the 99th percentile (MUFU rsqrt vs
1/sqrtf and summation order), restating tests/test_spatial_hash.cpp.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import vec_rel_err

pytestmark = pytest.mark.gpu


def _run(nb, s, cell=2.0, cutoff=2.0, eps=0.01, G=1.0, count=True):
    calc = nb.SpatialHashCalculator(cell, cutoff)
    calc.setGravitationalConstant(G)
    calc.setSofteningParameter(eps)
    if count:
        calc.set_flags(nb.FLAG_SYNC | nb.FLAG_COUNT_INTERACTIONS)
    n = len(s["x"])
    with nb.ScopedParticleData(n, {"pos_x": s["x"], "pos_y": s["y"], "pos_z": s["z"],
                                   "mass": s["m"]}) as p:
        calc.computeForces(p.device)
        p.download()
        acc = (p.host["acc_x"].copy(), p.host["acc_y"].copy(), p.host["acc_z"].copy())
    cells = calc.cell_data(n)
    nbrs = calc.interaction_counts(n) if count else None
    calc.close()
    return acc, cells, nbrs


def _cube(n, density=1.024, seed=3):
    side = (n / density) ** (1.0 / 3.0)
    return _uniform(n, side, seed)


def _uniform(n, side, seed):
    rng = np.random.default_rng(seed)
    s = {k: (rng.random(n) * side).astype(np.float32) for k in ("x", "y", "z")}
    s["m"] = np.full(n, 1.0 / n, np.float32)
    return s


def test_cutoff_boundary(nb):
    # tests/test_spatial_hash.cpp:81-127
    for r, zero in ((2.25, True), (1.75, False)):
        s = dict(x=np.array([0.0, r], np.float32), y=np.zeros(2, np.float32),
                 z=np.zeros(2, np.float32), m=np.ones(2, np.float32))
        (ax, ay, az), _, nbrs = _run(nb, s, 2.0, 2.0, 0.01, 1.0)
        if zero:
            assert ax[0] == 0.0 and ay[0] == 0.0 and az[0] == 0.0 and ax[1] == 0.0
            assert nbrs.tolist() == [0, 0]
        else:
            d2 = r * r + 1e-4
            exp = r / (d2 * np.sqrt(d2))
            assert abs(ax[0] - exp) < 1e-4 and abs(ax[1] + exp) < 1e-4
            assert nbrs.tolist() == [1, 1]


@pytest.mark.parametrize("n", [1, 2, 3, 100, 257, 5000, 60000])
def test_grid_and_neighbours_bit_exact(nb, orc, n):
    s = _cube(n, seed=n)
    (ax, ay, az), cells, nbrs = _run(nb, s)
    g = orc.hash_build(s["x"], s["y"], s["z"], 2.0)
    np.testing.assert_array_equal(cells["dims"], g["dims"])
    np.testing.assert_array_equal(cells["bmin"].view(np.uint32), g["bmin"].view(np.uint32))
    assert cells["total_cells"] == len(g["cell_start"])
    np.testing.assert_array_equal(cells["cell_start"], g["cell_start"])
    np.testing.assert_array_equal(cells["cell_end"], g["cell_end"])
    np.testing.assert_array_equal(cells["particle_cell"], g["particle_cell"])
    np.testing.assert_array_equal(cells["sorted_indices"], g["sorted_indices"])
    ox, oy, oz, onb = orc.hash_forces(g, s["x"], s["y"], s["z"], s["m"], 2.0, 1.0, 0.01)
    np.testing.assert_array_equal(nbrs, onb)
    if n > 1:
        has = onb > 0
        err = vec_rel_err(ax[has], ay[has], az[has], ox[has], oy[has], oz[has])
        if err.size:
            assert np.percentile(err, 99) <= 1e-5 and err.max() <= 1e-3
        assert np.all(ax[~has] == 0.0)


@pytest.mark.parametrize("clump", [40, 65, 3000])
def test_crowded_cells_match_oracle(nb, orc, clump):
    """A uniform cube plus a clump of `clump` bodies inside one cell (cells of
    very different sizes side by side): neighbour counts bit-exact, forces
    within the file's tolerance."""
    s = _cube(20000, seed=11)
    rng = np.random.default_rng(12)
    for k in ("x", "y", "z"):  # inside the cell [6, 8) of every axis
        s[k][:clump] = (6.2 + rng.random(clump) * 1.5).astype(np.float32)
    (ax, ay, az), cells, nbrs = _run(nb, s)
    sizes = cells["cell_end"] - cells["cell_start"]
    assert sizes.max() >= clump
    g = orc.hash_build(s["x"], s["y"], s["z"], 2.0)
    ox, oy, oz, onb = orc.hash_forces(g, s["x"], s["y"], s["z"], s["m"], 2.0, 1.0, 0.01)
    np.testing.assert_array_equal(nbrs, onb)
    has = onb > 0
    err = vec_rel_err(ax[has], ay[has], az[has], ox[has], oy[has], oz[has])
    assert np.percentile(err, 99) <= 1e-5 and err.max() <= 1e-3


def test_all_bodies_in_one_cell(nb, orc):
    # a cell larger than the system (as in a direct sum with a cutoff)
    s = _cube(3000, seed=13)
    (ax, ay, az), cells, nbrs = _run(nb, s, cell=1e3, cutoff=1e3)
    assert cells["total_cells"] == 8 and (cells["cell_end"] - cells["cell_start"]).max() == 3000
    g = orc.hash_build(s["x"], s["y"], s["z"], 1e3)
    ox, oy, oz, onb = orc.hash_forces(g, s["x"], s["y"], s["z"], s["m"], 1e3, 1.0, 0.01)
    np.testing.assert_array_equal(nbrs, onb)
    err = vec_rel_err(ax, ay, az, ox, oy, oz)
    assert np.percentile(err, 99) <= 1e-5 and err.max() <= 1e-3


def test_every_particle_in_exactly_one_cell(nb):
    # tests/test_spatial_hash.cpp:133-167 (several cell sizes)
    rng = np.random.default_rng(0)
    s = {k: rng.uniform(-10, 10, 50).astype(np.float32) for k in ("x", "y", "z")}
    s["m"] = np.ones(50, np.float32)
    for cell in (0.6, 1.0, 2.0, 5.5, 9.9):
        _, cells, _ = _run(nb, s, cell, min(cell, 0.5))
        seen = np.concatenate([cells["sorted_indices"][a:b] for a, b in
                               zip(cells["cell_start"], cells["cell_end"])])
        assert sorted(seen.tolist()) == list(range(50))


def test_cutoff_larger_than_cell_uses_cutoff(nb, orc):
    # SpatialHashCalculator::computeForces: effective cell = max(cell, cutoff)
    s = _cube(3000, seed=5)
    (ax, _, _), cells, nbrs = _run(nb, s, cell=1.0, cutoff=2.5)
    assert cells["cell"] == np.float32(2.5)
    g = orc.hash_build(s["x"], s["y"], s["z"], 2.5)
    _, _, _, onb = orc.hash_forces(g, s["x"], s["y"], s["z"], s["m"], 2.5, 1.0, 0.01)
    np.testing.assert_array_equal(nbrs, onb)


def test_grid_too_large_raises(nb):
    s = dict(x=np.array([0.0, 1e6], np.float32), y=np.array([0.0, 1e6], np.float32),
             z=np.array([0.0, 1e6], np.float32), m=np.ones(2, np.float32))
    with pytest.raises(nb.CapacityError, match="too large"):
        _run(nb, s, 1.0, 1.0)


@pytest.mark.slow
def test_full_size_uniform_cube(nb, orc):
    # The spatial-hash workload: N = 4,194,304 uniform in [0,160)^3, m = 1/N,
    # rc = cell = 2.0, eps = 0.01.  Grid arrays bit-exact; neighbour counts
    # bit-exact and forces within tolerance on 4096 seeded targets.
    s = nb.ics.uniform_cube(4_194_304, seed=3)
    (ax, ay, az), cells, nbrs = _run(nb, s)
    g = orc.hash_build(s["x"], s["y"], s["z"], 2.0)
    assert tuple(g["dims"]) == (82, 82, 82)
    for k in ("cell_start", "cell_end", "particle_cell", "sorted_indices"):
        np.testing.assert_array_equal(cells[k], g[k])
    t = np.random.default_rng(11).choice(len(s["x"]), 4096, replace=False)
    ox, oy, oz, onb = orc.hash_forces(g, s["x"], s["y"], s["z"], s["m"], 2.0, 1.0, 0.01,
                                      targets=t)
    np.testing.assert_array_equal(nbrs[t], onb)
    assert 30 < onb.mean() < 38  # ~34 neighbours within rc
    err = vec_rel_err(ax[t], ay[t], az[t], ox, oy, oz)
    assert np.percentile(err, 99) <= 1e-5


def test_grid_setup_matches_reference_fixture(nb, golden):
    # padded box and dims as the reference's own SpatialHashGrid::build host
    # code computed them (tests/golden/ref_grids.npz, made by make_golden.py)
    g = golden("ref_grids.npz")
    for name in g["names"]:
        p = g[f"{name}_p"]
        cell = float(g[f"{name}_cell"])
        s = {"x": p[:, 0].copy(), "y": p[:, 1].copy(), "z": p[:, 2].copy(),
             "m": np.full(len(p), 1.0 / len(p), np.float32)}
        _, cells, _ = _run(nb, s, cell, cell)
        np.testing.assert_array_equal(cells["dims"], g[f"{name}_dims"], err_msg=name)
        np.testing.assert_array_equal(cells["bmin"].view(np.uint32),
                                      g[f"{name}_bmin"].view(np.uint32), err_msg=name)
        assert cells["total_cells"] == int(g[f"{name}_total"]), name
