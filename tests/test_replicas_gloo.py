"""The multi-GPU row is replicas only: N independent runs, one per GPU, a barrier around
the timed region and the slowest rank's time. This checks bench.py's rank logic with two
gloo ranks on the CPU (no GPU involved)."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = bench.dist_env()
    dist.barrier()
    el = bench.max_over_ranks(torch, 1.0 + rank, w, "cpu")  # rank 1 is the slow one
    out[rank] = (r, w, lr, el, bench.replica_throughput(100.0, 10, w, el))
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_time():
    world = 2
    port = 29500 + (os.getpid() % 1000)
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][:3] == (0, 2, 0) and res[1][:3] == (1, 2, 1)
    for r in range(world):
        assert res[r][3] == 2.0                      # max over ranks
        assert res[r][4] == 100.0 * 10 * 2 / 2.0     # whole-job throughput of both replicas
