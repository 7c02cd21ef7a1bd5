"""Multi-process host logic of bench.py on CPU: two gloo ranks, max-over-ranks timing."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    w, r, local, pg = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(pg)
    v = bench.allreduce_max(pg, float(10 + rank))
    out[rank] = v
    pg.destroy_process_group()


def test_two_rank_max_timing():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn")
    assert dict(out) == {0: 11.0, 1: 11.0}
