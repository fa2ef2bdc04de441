"""The benchmark's multi-rank path on CPU: two gloo ranks on 127.0.0.1.

Worlds shard across ranks with no data-path exchange (weak scaling); the process group only
carries the barrier and the max/sum reductions of the timing. This checks that plumbing and
that each rank builds its own world mix (rank-specific seeds).
"""
import argparse
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    d = bench.Dist()
    d.barrier()
    mx = d.max(float(rank + 1))
    sm = d.sum(float(rank + 1))
    args = argparse.Namespace(workload="world_mix", worlds=8)
    worlds, cfg = bench.build_worlds(args, d.rank)
    first = worlds[0].pos[:4].copy()
    d.barrier()
    out.put((rank, mx, sm, cfg["seed"], cfg["bodies"], first))
    d.td.destroy_process_group()


def test_two_gloo_ranks_reduce_and_shard_worlds():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort(key=lambda x: x[0])
    for _, mx, sm, *_ in res:
        assert mx == 2.0 and sm == 3.0
    # each rank draws its own worlds (weak scaling: same per-rank size, different seed)
    assert res[0][3] != res[1][3]
    assert not np.array_equal(res[0][5], res[1][5])


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the CPU path the GPU arm is compared with) prints one JSON line
    with the arm's keys, its copies declared as zero, on a small sample."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "1", "--worlds", "8", "--cpu-sample", "2", "--cpu-seconds", "0.5"],
                       capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "dtype",
              "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
