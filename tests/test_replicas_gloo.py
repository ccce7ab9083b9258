"""The multi-GPU form of the bench is replicas only (independent processes, no data-path
collective): the whole-job number is world solves per the slowest rank's step time.
That host logic (bench.replicas_throughput) runs here as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, ms_by_rank, out):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    try:
        out.put((rank,) + bench.replicas_throughput(ms_by_rank[rank], world, "cpu"))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replicas_throughput_takes_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    ms = [10.0, 12.5]
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, ms, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms_max, value in res:
        assert ms_max == 12.5 and value == pytest.approx(2 * 1e3 / 12.5)


def test_replicas_throughput_single_process():
    sys.path.insert(0, REPO)
    import bench
    assert bench.replicas_throughput(8.0, 1) == (8.0, 125.0)
