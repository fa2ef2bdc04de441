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
