"""The N>1 bench path on CPU: two gloo ranks reduce their figures into the
whole-job line (moves of all ranks over the slowest rank's time)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    moves = 1000 * (rank + 1)          # 1000 and 2000 trial moves
    total_ms = 10.0 * (rank + 1)       # 10 and 20 ms
    value, e2e, ms = bench.reduce_over_ranks(moves, total_ms, 500 * (rank + 1), 0.5 * (rank + 1), world, "cpu")
    out.put((rank, value, e2e, ms))
    dist.destroy_process_group()


def test_two_gloo_ranks_sum_work_over_slowest_time():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = 29400 + os.getpid() % 1000
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, e2e, ms in res:
        assert ms == 20.0
        assert value == pytest.approx(3000 / 0.020)
        assert e2e == pytest.approx(1500 / 1.0)


def test_single_rank_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench

    value, e2e, ms = bench.reduce_over_ranks(1000, 10.0, 500, 0.5, 1, "cpu")
    assert value == pytest.approx(1e5) and e2e == pytest.approx(1000) and ms == 10.0
