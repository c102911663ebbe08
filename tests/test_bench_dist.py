"""The multi-rank path of the benchmark (replicas: the barrier, the max of the
timings over ranks and the whole-job rate) with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    import bench
    w, r, local, dist = bench.dist_setup("gloo")
    assert (w, r, local) == (world, rank, rank)
    dist.barrier()
    t = bench.max_over_ranks(1.0 + rank, dist)          # rank 1 is the slow one
    out[rank] = (t, bench.replica_rate(w, 1000, 5, t))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert out[0] == out[1] == (2.0, 2 * 1000 * 5 / 2.0)


def test_single_process_needs_no_collectives():
    import bench
    assert bench.dist_setup()[0] == int(os.environ.get("WORLD_SIZE", "1"))
    assert bench.max_over_ranks(3.5, None) == 3.5
