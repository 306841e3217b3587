"""The multi-GPU path of bench.py on the CPU: the solve does not shard, so
under torchrun every rank runs an independent replica and the job's time per
step is the slowest rank's.  Two gloo ranks check the reduction and the
environment parsing."""
import os
import sys

import pytest
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_env() == (rank, rank, world)
    got = bench.replica_max([10.0 + rank, 5.0 - rank], dist, "cpu")
    out.put((rank, got))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=90) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert res[0] == res[1] == [11.0, 5.0]


def test_single_process_is_identity():
    sys.path.insert(0, REPO)
    import bench
    assert bench.replica_max([3.5, 7.25]) == [3.5, 7.25]
