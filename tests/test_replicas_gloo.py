"""Multi-process path of bench.py on CPU (gloo, world size 2).

Independent scenes shard across GPUs without any collective on the data path:
every rank computes the same balanced partition of the batch's scenes and
takes its own disjoint share; the step time is the maximum over ranks and the
whole-job rate counts every rank's cells (summed over ranks).  Single scenes
do not shard (replicas only)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "incremental-fluids_gb300")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path[:0] = [ROOT, PKG]
    import torch
    import torch.distributed as dist
    import bench
    from ifluids import scenes
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 100.0 * (rank + 1)  # rank 1 is the slow one
    t = bench.max_over_ranks(local_ms, world)
    rate = bench.whole_job_rate(1000.0, 5, world, t)
    # the batch's partition: the generator's first 512 x world scenes, disjoint shares
    allscs = scenes.batch_scenes(count=512 * world, seed=2)
    work = [bench.scene_work(s.w, s.h) for s in allscs]
    mine = bench.shard_scenes(work, rank, world)
    cells = sum(allscs[i].cells for i in mine)
    cells_all = bench.sum_over_ranks(float(cells), world)
    shares = [None] * world
    dist.all_gather_object(shares, mine)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, rate, cells_all, shares, sum(work[i] for i in mine), sum(work),
           sum(s.cells for s in allscs)))


def test_max_over_ranks_rate_and_disjoint_shards():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, rate, cells_all, shares, my_work, all_work, all_cells in out:
        assert t == 200.0                        # both ranks see the slowest rank's time
        assert rate == 2 * 1000.0 * 5 / 0.2       # every rank's cells, over the slowest time
        assert cells_all == all_cells            # the summed shares cover every scene's cells
        a, b = set(shares[0]), set(shares[1])
        assert not (a & b) and a | b == set(range(1024))  # disjoint and complete
        assert abs(my_work / all_work - 0.5) < 0.01       # balanced by estimated work
    assert out[0][4] == out[1][4]                # every rank computed the same partition


def test_single_rank_is_identity():
    sys.path[:0] = [ROOT]
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.sum_over_ranks(3.0, 1) == 3.0
    assert bench.whole_job_rate(10.0, 2, 1, 1000.0) == 20.0
    assert bench.shard_scenes([3.0, 1.0, 2.0], 0, 1) == [0, 1, 2]
