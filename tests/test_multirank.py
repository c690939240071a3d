"""The multi-GPU path of bench.py is replicas only: every rank runs its own
batch of independent trajectories (same recipe, own seeds) with no
collective on the data path; the job's time is the maximum over ranks.  Two
gloo ranks on the CPU check that host logic."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as tmp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    from qsource_gb300 import synth
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    # a small member of each rank's batch: a window and a replica
    w = synth.lambda_batch_member(3, nwindows=5, replicas=2, rank=rank)
    r = synth.lambda_batch_member(5, nwindows=5, replicas=2, rank=rank)
    ms = bench.max_over_ranks(dist, 10.0 + rank)
    out[rank] = (w.natom, r.natom, float(w.x.sum()), float(r.x.sum()), ms)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_run_independent_replicas():
    world = 2
    port = _free_port()
    mgr = tmp.Manager()
    out = mgr.dict()
    tmp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
    a, b = out[0], out[1]
    assert a[2] != b[2] and a[3] != b[3]          # own seeds: different coordinates
    assert a[4] == b[4] == 11.0                   # the job time is the slowest rank's
    import bench
    assert bench.aggregate_ns_per_day(2, 32, 100, 50.0) == pytest.approx(2 * bench.aggregate_ns_per_day(1, 32, 100, 50.0))
