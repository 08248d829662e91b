"""The multi-GPU path of the benchmark is replicas only (one GPU per rank,
no data exchange).  Its host logic runs here as two gloo ranks on the CPU:
the barrier, the slowest-rank time and the whole-job value."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    ms = bench.max_over_ranks(world, 100.0 + 25.0 * rank)  # rank 1 is the slow replica
    out.put((rank, ms, bench.replica_value(world, 512 ** 3, 300, ms)))
    bench.barrier(world)
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_whole_job():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [125.0, 125.0]
    want = 2 * 512 ** 3 * 300 / 0.125 / 1e9
    assert all(abs(r[2] - want) < 1e-9 * want for r in res)
