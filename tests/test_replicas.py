"""Replica sharding of a sweep over ranks (gloo, world size 2, CPU): every
system is integrated by exactly one rank, and the per-rank results combine to
the single-process result.  The GPU bench uses the same shard function; there
is no data-path collective (systems are independent)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import systems


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def worker(rank, world, port, out):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "oracle"))
    sys.path.insert(0, os.path.join(root, "p9-integrator_gb300"))
    import torch

    from oracle import Oracle
    from oracle import default_params as oparams

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    full = systems.sweep(n_systems=6, nt_lo=8, nt_hi=20, seed=3)
    mine = systems.shard(full, rank, world)
    O = Oracle()
    O.set_threads(1)
    p = oparams(dt=0.5, hill_factor=3.0, drift=1)
    pos, vel, alag = O.load_elements(p, mine.body_offset, mine.n_massive, mine.mass, mine.elements)
    pos, vel, *_ = O.run(p, mine.body_offset, mine.n_massive, mine.mass, pos, vel, alag, steps=5)
    # body counts summed over ranks, as bench.py sums its replicas' work
    t = torch.tensor([float(mine.n_total)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    out[rank] = (pos, float(t.item()), mine.n_systems)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sweep_matches_single_process():
    world = 2
    port = free_port()
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(worker, args=(world, port, out), nprocs=world, join=True)
    full = systems.sweep(n_systems=6, nt_lo=8, nt_hi=20, seed=3)
    assert out[0][1] == out[1][1] == float(full.n_total)
    assert out[0][2] + out[1][2] == full.n_systems
    # single process reference
    import sys

    from oracle import Oracle
    from oracle import default_params as oparams

    O = Oracle()
    p = oparams(dt=0.5, hill_factor=3.0, drift=1)
    pos, vel, alag = O.load_elements(p, full.body_offset, full.n_massive, full.mass, full.elements)
    pos, *_ = O.run(p, full.body_offset, full.n_massive, full.mass, pos, vel, alag, steps=5)
    n0 = int(systems.shard(full, 0, world).n_total)
    ref = pos.reshape(3, -1)
    got = np.concatenate([out[0][0].reshape(3, -1), out[1][0].reshape(3, -1)], axis=1)
    assert np.array_equal(got, ref)
    assert got.shape[1] == full.n_total and n0 > 0
