"""The N-GPU bench path on CPU ranks: two processes over the gloo backend agree on the job's
timed totals (the slowest rank's) and on the whole-job rate, as bench.py computes them
under torchrun (the GPU run uses NCCL; the reduction and the arithmetic are the same)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = [10.0 + 5.0 * rank, 20.0 - 3.0 * rank]  # per-rank totals (ms) of 4 steps
    tot, tot_e2e = bench.job_totals(mine, dist, "cpu")
    out[rank] = (tot, tot_e2e, bench.job_rate(world, 4, tot))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_job_totals_and_rate():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world, port = 2, 29517 + os.getpid() % 1000
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        tot, tot_e2e, rate = res[r]
        assert tot == 15.0 and tot_e2e == 20.0  # the maximum over the ranks
        assert rate == pytest.approx(world * 4 / 0.015)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_totals([3.0, 4.0]) == [3.0, 4.0]
    assert bench.job_rate(1, 10, 2000.0) == pytest.approx(5.0)
