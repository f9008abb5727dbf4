"""The multi-rank host path of bench.py with world_size 2 on the gloo backend (CPU): each
rank builds its own walker batch, the step time is the maximum over ranks, the whole-job
rate counts every rank's packets, and only rank 0 runs the reference arm."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import argparse

    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    args = argparse.Namespace(workload="batched", models=3, seed=0, packets=1000)
    models = bench.build_models(args, rank)
    masses = [m.params["mass"] for m in models]
    t = bench.max_over_ranks(100.0 + 50.0 * rank, world)
    rate = bench.weak_scaling_rate(world, 3 * 1000, 1, t)
    # reference arm: rank 1 must return without work
    ref = None
    if rank == 1:
        ref = bench.run_reference(argparse.Namespace(), world, rank)
    out[rank] = (masses, t, rate, ref)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shard_walkers_and_take_the_slowest_time():
    world = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world,
                       start_method="spawn", join=True)
    m0, t0, r0, _ = out[0]
    m1, t1, r1, ref = out[1]
    assert len(m0) == len(m1) == 3 and not np.allclose(m0, m1)   # independent walkers
    assert t0 == t1 == 150.0                                     # max over ranks
    assert r0 == r1 == 2 * 3000 / 0.150                           # whole-job rate
    assert ref is None
