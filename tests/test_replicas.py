"""Multi-GPU runs are independent replicas (no exchange step on one problem
per GPU): the bench reduces the ranks' times with a MAX all-reduce and
reports all ranks' units over the slowest time.  Checked here with two gloo
ranks on the CPU."""
import os
import socket
import sys

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    t = 1.0 + rank  # rank 1 is the slow one
    t_max = bench.max_over_ranks(t, w, "cpu")
    value = bench.replica_value(100.0, t_max, w)
    dist.barrier()
    out[rank] = (t_max, value)
    dist.destroy_process_group()


def test_replica_timing_two_gloo_ranks():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (2.0, 100.0)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.replica_value(10.0, 2.0, 1) == 5.0
