"""Multi-GPU is replicas only: each rank advances its own replica set and the
ranks meet only for the timing barrier and the max over ranks of the timed
region (bench.py's dist helpers).  Checked here with world_size 2 on the gloo
backend (CPU), the rendezvous on 127.0.0.1."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    w, r = bench.dist_setup()
    assert (w, r) == (world, rank)
    bench.dist_barrier(w)
    out[rank] = bench.dist_max(float(10 + 5 * rank), w)
    # replica seeds differ per rank: independent units, no data-path exchange
    e = bench.random_state(1, 8, seed=7 + rank)
    out[world + rank] = float(e[0, 0, 0])
    import torch.distributed as dist
    dist.destroy_process_group()


def test_max_over_ranks_and_independent_replicas():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    assert out[0] == out[1] == 15.0
    assert out[2] != out[3]
