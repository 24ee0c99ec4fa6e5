"""The multi-GPU form of the bench is replicas only: each rank runs its own
scene, and the ranks meet only to agree on the job's time (the slowest
rank's) before rank 0 reports the whole job's particle-steps per second.
That host-side aggregation runs here on CPU with two gloo ranks."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local, dist = bench.dist_setup(world)
    assert (r, w, local) == (rank, world, rank) and dist is not None
    ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
    bench.barrier(dist)
    job_ms = bench.max_over_ranks(dist, ms)
    out[rank] = (job_ms, bench.whole_job_value(w, 1000, 4, job_ms))
    dist.destroy_process_group()


def test_two_replicas_agree_on_the_slowest_rank():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    job_ms, value = res[0]
    assert job_ms == 15.0
    assert value == pytest.approx(world * 1000 * 4 / 0.015)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, 3.5) == 3.5
    assert bench.whole_job_value(1, 1000, 2, 1.0) == pytest.approx(2e6)
