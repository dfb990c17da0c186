"""The bench's multi-replica path on CPU: two gloo ranks, each one replica of the workload.
The whole-job figure takes the slowest rank's time and the particle-steps of all ranks;
there is no collective on the data path."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ms, psteps = bench.aggregate_over_ranks(10.0 + 5.0 * rank, 1000 * (rank + 1), "cpu")
    out[rank] = (ms, psteps)
    dist.destroy_process_group()


def test_two_replicas_gloo():
    world = 2
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        assert res[r] == (15.0, 3000.0)
