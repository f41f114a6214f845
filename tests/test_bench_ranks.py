"""bench.py's multi-GPU arithmetic (independent replicas, one per rank): the timed region is
the maximum over the ranks and the whole-job value counts every rank's walker-steps.
Two gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.5 + rank, dist, "cpu")
        out[rank] = (t, bench.replica_throughput(3, world, t))
    finally:
        dist.destroy_process_group()


def test_two_ranks_max_time_and_whole_job_value():
    mp = pytest.importorskip("torch.multiprocessing")
    import bench
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
    assert res[0][0] == res[1][0] == 2.5
    want = bench.WALKERS * (bench.BURN + bench.RUN) * 3 * 2 / 2.5
    assert res[0][1] == res[1][1] == pytest.approx(want)


def test_one_rank_is_unchanged():
    import bench
    assert bench.max_over_ranks(4.0, None, "cpu") == 4.0
    assert bench.replica_throughput(1, 1, 2.0) == bench.WALKERS * (bench.BURN + bench.RUN) / 2.0
