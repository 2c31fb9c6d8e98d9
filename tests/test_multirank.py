"""Multi-rank host logic on CPU (gloo, world size 2): each rank runs its own
lattice (replicas, weak scaling) and the job's time is the maximum over the
ranks, as bench.py does under torchrun with NCCL.  The lattice work here is
the CPU oracle; no GPU is involved."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from oracle import oracle as O
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    assert (ws, r, local) == (world, rank, rank)
    # replica of the workload on a small lattice, seed per rank as in bench.py
    seed = 2 + 1000 * r
    W, H = 128, 64
    from lgca_gb300 import geometry as G
    types = G.disc(W, H, 16, 32, 8)
    st = O.init_bernoulli(3, W, H, types, seed=seed, p_move=0.3, p_rest=0.3)
    fin = O.run(3, st, 10, types=types, seed=seed, force_x=4, force_p=0.02)
    n = torch.tensor([float(O.count_particles(fin))])
    t = torch.tensor([0.1 * (r + 1)])  # per-rank time
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total = n.clone()
    dist.all_reduce(total, op=dist.ReduceOp.SUM)
    out[rank] = (float(t.item()), float(total.item()), float(n.item()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_max_time_and_totals():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    assert out[0][0] == pytest.approx(0.2) and out[1][0] == pytest.approx(0.2)
    assert out[0][1] == out[1][1] == out[0][2] + out[1][2]
    # independent seeds give independent replicas
    assert out[0][2] != out[1][2]
