"""Replica aggregation of bench.py under torch.distributed (gloo, 2 ranks on CPU): the
whole-job rate is the particles of all ranks over the slowest rank's time."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = 100.0 + 50.0 * rank  # rank 1 is the slow replica
    slowest = bench.max_over_ranks(ms, "cpu")
    out.put((rank, slowest, bench.replica_rate(1000, 10, slowest, world)))
    torch.distributed.destroy_process_group()


def test_replicas_report_the_whole_job_over_the_slowest_rank():
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, rate in res:
        assert slowest == 150.0
        assert rate == pytest.approx(2 * 1000 * 10 / 0.150)
