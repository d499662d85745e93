"""The multi-GPU path of bench.py is replicas only (one independent box per
rank, no collective on the data path): two gloo ranks on the CPU check the
rendezvous, the barrier and the whole-job throughput (all ranks' updates
over the slowest rank's time)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), BENCH_BACKEND="gloo")
    import bench
    r, w, local, pg = bench.dist_setup()
    bench.barrier(pg)
    value, ms = bench.replica_throughput(pg, w, 1000, 10, 5.0 + r)  # rank 1 is the slower one
    out.put((r, w, value, ms))
    pg.destroy_process_group()


def test_two_gloo_ranks_report_whole_job_throughput():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, w, value, ms) in enumerate(res):
        assert (rank, w) == (r, world)
        assert ms == 6.0
        assert value == pytest.approx(world * 1000 * 10 / 6.0e-3, rel=1e-15)
