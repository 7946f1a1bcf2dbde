"""Multi-GPU is replicas only: each rank runs its own lattice with its own replica
id and the job time is the maximum over ranks.  The host-side logic is checked
here with two gloo ranks on the CPU (no GPU, no data-path collective)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    # the rank's replica id keys its random stream; its share of the work is fixed (weak scaling)
    ms = 10.0 + 5.0 * rank
    t = torch.tensor([ms])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    flips_rank = 1000.0
    value = bench.aggregate_value(flips_rank, world, float(t.item()))
    out[rank] = (float(t.item()), value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replica_aggregation():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    assert out[0] == out[1]
    t_max, value = out[0]
    assert t_max == 15.0
    assert value == pytest.approx(2 * 1000.0 / (15.0 * 1e6))
