"""The benchmark's multi-rank path on CPU (gloo, world size 2).

Every rank serves its own shard of the request stream (weak scaling); the
only collectives are the maximum of the elapsed time and the sum of the
particle-steps over ranks; the reference arm runs on rank 0 alone and the
other rank exits 0 without work.  Ranks rendezvous on 127.0.0.1.
"""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(script: str, *args, timeout=300):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), script, *args]
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""),
               CUDA_VISIBLE_DEVICES="")
    return subprocess.run(cmd, capture_output=True, text=True, timeout=timeout, cwd=ROOT, env=env)


def test_reduce_over_ranks_gloo(tmp_path):
    script = tmp_path / "ranks.py"
    script.write_text(
        "import json, os, sys\n"
        "import torch.distributed as dist\n"
        "import bench\n"
        "dist.init_process_group('gloo')\n"
        "r, w = dist.get_rank(), dist.get_world_size()\n"
        "t, ps = bench.reduce_over_ranks(1.0 + r, 100.0 * (r + 1), w)\n"
        "out = os.path.join(sys.argv[1], f'rank{r}.json')\n"
        "open(out, 'w').write(json.dumps({'rank': r, 't': t, 'ps': ps, 'seed': bench.shard_seed(r)}))\n"
        "dist.destroy_process_group()\n")
    res = _torchrun(str(script), str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    assert sorted(d["rank"] for d in lines) == [0, 1]
    for d in lines:
        assert d["t"] == 2.0 and d["ps"] == 300.0  # max of elapsed, sum of work
    assert len({d["seed"] for d in lines}) == 2  # disjoint request shards


def test_reference_arm_two_ranks():
    res = _torchrun(os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                    "--steps", "1", "--warmup", "0", "--ref-budget-s", "1")
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads(l) for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    d = lines[0]
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
