"""The multi-GPU path on the CPU: two gloo ranks, as bench.py runs one process per GPU.

Systems of an ensemble and jobs of a stream are independent, so N GPUs split them by
estimated cost with no exchange: every rank computes the same split locally.  The ranks only
meet for the barrier around the timed region and the max over ranks of the time.
"""
import os
import socket

import pytest

from lpmd2_gb300 import inputs as I
from lpmd2_gb300.serve import partition


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench

    r, w, _, dist = bench.dist_setup(world)
    jobs = I.job_stream(40, 100.0, seed=5)
    costs = [4 * j["k"] ** 3 * j["steps"] for j in jobs]
    mine = partition(costs, w)[r]
    gathered = [None] * w
    dist.all_gather_object(gathered, mine)
    slowest = bench.allmax(dist, float(10 * (r + 1)))
    bench.barrier(dist)
    q.put((r, gathered, slowest))
    dist.destroy_process_group()


def test_two_gloo_ranks_split_the_work_without_overlap():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        results = [q.get(timeout=180) for _ in procs]
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert sorted(r for r, _, _ in results) == [0, 1]
    for _, parts, slowest in results:
        assert slowest == 20.0
        assert sorted(parts[0] + parts[1]) == list(range(40))
        assert not set(parts[0]) & set(parts[1])
    assert results[0][1] == results[1][1]  # the same split on both ranks


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_covers_and_balances(world):
    costs = [4 * s["k"] ** 3 for s in I.job_stream(200, 50.0, seed=3)]
    parts = partition(costs, world)
    assert sorted(i for p in parts for i in p) == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) <= sum(costs) / world + max(costs)
    assert parts == partition(costs, world)
