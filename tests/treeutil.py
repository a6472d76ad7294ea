"""Canonical form of an octree in the reference's OctreeNode layout.

The reference numbers nodes in insertion order, the CUDA build in depth-first
pre-order; the tree itself (topology and every node's fields) is compared
after keying each node by its octant path from the root.
"""
from __future__ import annotations

import numpy as np


def canonical(nodes: np.ndarray) -> dict:
    """path tuple -> (is_leaf, particle_index, particle_count, mass, com, center, half) bits."""
    out = {}
    stack = [(0, ())]
    seen = 0
    while stack:
        idx, path = stack.pop()
        nd = nodes[idx]
        seen += 1
        key = (int(nd["is_leaf"]), int(nd["particle_index"]), int(nd["particle_count"]),
               np.float32(nd["mass"]).view(np.uint32).item(),
               tuple(np.asarray(nd["com"], np.float32).view(np.uint32).tolist()),
               tuple(np.asarray(nd["center"], np.float32).view(np.uint32).tolist()),
               np.float32(nd["half"]).view(np.uint32).item())
        assert path not in out, "node reached twice"
        out[path] = key
        for o in range(8):
            c = int(nd["children"][o])
            if c >= 0:
                stack.append((c, path + (o,)))
    assert seen == len(nodes), f"unreachable nodes: {len(nodes) - seen}"
    return out


def compare(a: np.ndarray, b: np.ndarray) -> list:
    """Differences between two trees (empty list when identical)."""
    ca, cb = canonical(a), canonical(b)
    diffs = []
    for p in sorted(set(ca) | set(cb)):
        if ca.get(p) != cb.get(p):
            diffs.append((p, ca.get(p), cb.get(p)))
            if len(diffs) > 10:
                break
    return diffs
