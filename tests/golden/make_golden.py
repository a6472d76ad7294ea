"""Generate the golden fixtures in this directory from the reference's own code.

Run in a checkout where the reference sources exist (they are compiled in
place into oracle/_ref by oracle/build.py; nothing is copied):

    python tests/golden/make_golden.py

Every fixture is produced by calling the reference's host code through
oracle/_ref/libnbody_ref.so (ref_harness.cpp):
  * ref_inputs.npz    -- ParticleInitializer::initSpherical / initUniform
                         outputs (std::mt19937 seed 42) for the reference's
                         own test scenarios, plus the deterministic N=32 grid
                         of tests/test_force_calculation.cpp:117-121;
  * ref_pair.npz      -- computeGravitationalAccelerationCPU on seeded pairs;
  * ref_morton.npz    -- computeMortonCode on seeded and edge coordinates;
  * ref_cells.npz     -- SpatialHashGrid::getCellIndex on seeded points;
  * ref_grids.npz     -- SpatialHashGrid::build's padded bounding box and
                         grid dimensions (run on the host up to its first
                         cell kernel) for seeded and edge point sets;
  * ref_trees.npz     -- BarnesHutTree::buildTreeOnHost node arrays for
                         several inputs (Morton-sorted with a stable sort);
  * ref_checkpoint.nbody -- Serializer::save of a small state.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle.oracle import Oracle, Reference  # noqa: E402


def main() -> None:
    ref = Reference()
    orc = Oracle()  # only for the bbox / key order fed to the reference tree build
    rng = np.random.Generator(np.random.PCG64(20240607))

    # --- inputs of the reference's own tests ---------------------------------
    inputs = {}
    for n, radius in ((30, 5.0), (50, 10.0), (50, 5.0), (100, 10.0), (100, 5.0)):
        s = ref.init_spherical(n, radius=radius, seed=42)
        for k, v in s.items():
            inputs[f"sph{n}_r{int(radius)}_{k}"] = v
    for n, lo, hi in ((100, -10.0, 10.0), (100, -5.0, 5.0), (50, -10.0, 10.0)):
        s = ref.init_uniform(n, [lo] * 3, [hi] * 3, seed=42)
        for k, v in s.items():
            inputs[f"uni{n}_{int(hi)}_{k}"] = v
    i = np.arange(32)
    inputs["grid32_x"] = ((i * 7) % 11).astype(np.float32) * np.float32(0.3)
    inputs["grid32_y"] = ((i * 3) % 13).astype(np.float32) * np.float32(0.3)
    inputs["grid32_z"] = ((i * 5) % 9).astype(np.float32) * np.float32(0.3)
    inputs["grid32_m"] = np.float32(0.5) + np.float32(0.1) * (i % 5).astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "ref_inputs.npz"), **inputs)

    # --- pair function -------------------------------------------------------
    k = 2000
    p1 = rng.uniform(-10, 10, (k, 3)).astype(np.float32)
    p2 = (p1 + rng.normal(0, 2, (k, 3))).astype(np.float32)
    p2[:10] = p1[:10]  # coincident pairs
    m2 = rng.uniform(0.01, 100, k).astype(np.float32)
    eps = rng.choice(np.array([0.0, 0.001, 0.01, 0.1, 1.0], np.float32), k)
    eps[:10] = np.float32(0.1)
    G = rng.choice(np.array([1.0, 6.674e-3, 2.5], np.float32), k)
    acc = np.stack([ref.pair_accel(p1[j], p2[j], m2[j], G[j], eps[j]) for j in range(k)])
    np.savez_compressed(os.path.join(HERE, "ref_pair.npz"), p1=p1, p2=p2, m2=m2, eps=eps, G=G,
                        acc=acc)

    # --- Morton codes ----------------------------------------------------------
    nx = rng.uniform(-0.2, 1.2, (5000, 3)).astype(np.float32)
    edge = np.array([0.0, 1.0, 0.5, 1 / 1023, 2 / 1023, np.nextafter(np.float32(1), np.float32(0)),
                     -0.0, 1e-30, 0.9990234, 0.0009775], np.float32)
    e3 = np.stack(np.meshgrid(edge, edge, edge, indexing="ij"), -1).reshape(-1, 3)
    nx = np.concatenate([nx, e3]).astype(np.float32)
    codes = np.array([ref.morton_code(*v) for v in nx], np.uint32)
    np.savez_compressed(os.path.join(HERE, "ref_morton.npz"), n=nx, code=codes)

    # --- cell indices ----------------------------------------------------------
    pts = rng.uniform(-50, 50, (3000, 3)).astype(np.float32)
    cells = rng.choice(np.array([0.5, 1.0, 2.0, 3.7], np.float32), 3000)
    pts = np.concatenate([pts, np.array([[0.5, 0.5, 0.5], [2.5, 4.5, 6.5], [-0.0, 2.0, -2.0]],
                                        np.float32)])
    cells = np.concatenate([cells, np.array([2.0, 2.0, 2.0], np.float32)])
    ci = np.array([ref.cell_index(*pts[j], cells[j]) for j in range(len(pts))], np.int32)
    np.savez_compressed(os.path.join(HERE, "ref_cells.npz"), p=pts, cell=cells, idx=ci)

    # --- hash grid setup: padded box and dims (SpatialHashGrid::build) ---------
    grids = {}
    gcases = []
    for j, (lo, hi, n, cell) in enumerate([(0, 160, 3000, 2.0), (-50, 50, 3000, 3.7),
                                          (-1e3, 1e3, 2000, 25.0), (0, 10, 1500, 0.5),
                                          (-3, 7, 1000, 1.0), (1e4, 1e4 + 64, 1000, 2.0)]):
        p = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
        gcases.append((f"u{j}", p, np.float32(cell)))
    # edge sets: extents that are exact multiples of the cell, one point,
    # coincident points, a flat slab, coordinates on cell boundaries
    gcases.append(("grid_pts", np.stack(np.meshgrid(*[np.arange(0, 20, 2.0)] * 3),
                                        -1).reshape(-1, 3).astype(np.float32), np.float32(2.0)))
    gcases.append(("one", np.array([[1.5, -2.5, 3.0]], np.float32), np.float32(1.0)))
    gcases.append(("coincident", np.full((64, 3), 4.0, np.float32), np.float32(0.25)))
    slab = rng.uniform(-8, 8, (500, 3)).astype(np.float32)
    slab[:, 2] = 0.5
    gcases.append(("slab", slab, np.float32(0.8)))
    names = []
    for name, p, cell in gcases:
        g = ref.hash_grid_setup(p[:, 0], p[:, 1], p[:, 2], cell)
        grids[f"{name}_p"] = p
        grids[f"{name}_cell"] = cell
        grids[f"{name}_bmin"] = g["bmin"]
        grids[f"{name}_bmax"] = g["bmax"]
        grids[f"{name}_dims"] = g["dims"]
        grids[f"{name}_total"] = np.int64(g["total_cells"])
        names.append(name)
    # a grid the reference rejects (more than 1e8 cells)
    big = np.array([[0.0, 0.0, 0.0], [1000.0, 1000.0, 1000.0]], np.float32)
    try:
        ref.hash_grid_setup(big[:, 0], big[:, 1], big[:, 2], np.float32(2.0))
        rejected = False
    except OverflowError:
        rejected = True
    grids["too_large_p"] = big
    grids["too_large_cell"] = np.float32(2.0)
    grids["too_large_rejected"] = np.bool_(rejected)
    grids["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "ref_grids.npz"), **grids)

    # --- octrees built by the reference's host insertion -------------------
    trees = {}
    cases = {
        "sph30": ref.init_spherical(30, radius=5.0, seed=42),
        "sph100": ref.init_spherical(100, radius=10.0, seed=42),
        "sph700": ref.init_spherical(700, radius=10.0, seed=7),
        "uni500": ref.init_uniform(500, [-10] * 3, [10] * 3, seed=9),
    }
    coinc = {k: np.zeros(16, np.float32) for k in ("x", "y", "z", "vx", "vy", "vz")}
    coinc["x"][:], coinc["y"][:], coinc["z"][:] = 1.0, 2.0, 3.0
    coinc["m"] = np.ones(16, np.float32)
    cases["coincident16"] = coinc
    line = {k: np.zeros(16, np.float32) for k in ("x", "y", "z", "vx", "vy", "vz")}
    line["x"] = (np.float32(0.0001) * np.arange(16, dtype=np.float32)).astype(np.float32)
    line["m"] = np.ones(16, np.float32)
    cases["collinear16"] = line
    for name, s in cases.items():
        bmin, bmax = orc.bbox(s["x"], s["y"], s["z"])
        keys, idx = orc.morton_keys(s["x"], s["y"], s["z"], bmin, bmax)
        ks, si = orc.stable_sort(keys, idx)
        nodes, depth = ref.build_tree(s["x"], s["y"], s["z"], s["m"], si, bmin, bmax)
        for k2 in ("x", "y", "z", "m"):
            trees[f"{name}_{k2}"] = s[k2]
        trees[f"{name}_keys"] = ks
        trees[f"{name}_sorted"] = si
        trees[f"{name}_nodes"] = np.frombuffer(nodes.tobytes(), np.uint8)
        trees[f"{name}_depth"] = np.int32(depth)
    np.savez_compressed(os.path.join(HERE, "ref_trees.npz"), **trees)

    # --- checkpoint ----------------------------------------------------------------
    s = ref.init_spherical(7, radius=3.0, seed=42)
    s["vx"] = np.linspace(-1, 1, 7).astype(np.float32)
    ref.save_checkpoint(os.path.join(HERE, "ref_checkpoint.nbody"), s, sim_time=1.25, dt=0.002,
                        G=1.5, softening=0.05, method=2)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
