"""Multi-process path of bench.py on CPU (gloo, world size 2): every rank runs
an independent replica (scenes never exchange data), the step time is the
maximum over ranks and the whole-job rate counts every rank's cells."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 100.0 * (rank + 1)  # rank 1 is the slow one
    t = bench.max_over_ranks(local_ms, world)
    rate = bench.whole_job_rate(1000.0, 5, world, t)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, rate))


def test_max_over_ranks_and_whole_job_rate():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, rate in out:
        assert t == 200.0                        # both ranks see the slowest rank's time
        assert rate == 2 * 1000.0 * 5 / 0.2       # every rank's cells, over the slowest time


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.whole_job_rate(10.0, 2, 1, 1000.0) == 20.0
