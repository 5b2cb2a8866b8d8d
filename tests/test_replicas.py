"""The N-rank timing of bench.py: a barrier around the timed region and the
slowest rank's time (max over ranks), exercised with two gloo ranks on the CPU
(the sharded step itself is covered by tests/test_slabs.py)."""

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

    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench._dist = dist
    bench.barrier()
    ms = 10.0 + 5.0 * rank  # per-rank timed-region length
    out[rank] = bench.max_over_ranks(ms)
    bench.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
        assert dict(out) == {0: 15.0, 1: 15.0}
