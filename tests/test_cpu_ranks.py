"""The multi-GPU form of the benchmark on CPU: world_size 2 over gloo. Each rank culls its own frame
(replicas, no data-path collective); the job's time is the slowest rank's and its throughput every
rank's objects over that time. Here each rank runs the oracle on its own seeded shard."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from blitzen_gb300 import scenes as S
    from oracle import oracle as O
    from tests.helpers import view_for
    sc = S.frustum_lod_scene(5_000, seed=100 + rank)
    n, recs, _ = O.cull(0, view_for(zfar=1e30), sc)
    ms = 1.0 + rank  # rank 1 is the slow one
    t = bench.max_over_ranks(ms, world, "cpu")
    out[rank] = (t, bench.job_throughput(sc.count, world, t), n)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_report_the_slowest_and_the_job_total():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.0           # both ranks see the slowest time
    assert res[0][1] == pytest.approx(2 * 5_000 / 2e-3)
    assert res[0][2] > 0 and res[1][2] > 0          # each rank culled its own shard
