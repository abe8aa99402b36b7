"""The multi-process path of bench.py on CPU: two gloo ranks launched the way
torchrun launches them (RANK / WORLD_SIZE / MASTER_* in the environment).

The hot path does not shard (replicas only), so what N > 1 adds is the
rendezvous, the barrier around the timed region and the whole-job value from
the slowest rank's time; those are checked here without a GPU.
"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    r, ws, local, dist = bench.dist_setup(backend="gloo")
    assert (r, ws, local) == (rank, world, rank)
    bench.barrier(dist)
    # rank r "took" 1 + r seconds for 1000 cell-updates: the job's time is the slowest rank's
    slowest = bench.max_over_ranks(dist, 1.0 + rank)
    value = bench.replica_value(ws, 1000, slowest)
    bench.barrier(dist)
    out[rank] = (slowest, value)
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank_time():
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1] == (2.0, 1000.0)


def test_single_process_needs_no_rendezvous(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    sys.path.insert(0, ROOT)
    import bench

    assert bench.dist_setup() == (0, 1, 0, None)
    assert bench.max_over_ranks(None, 3.5) == 3.5
    assert bench.replica_value(1, 500, 2.0) == 250.0
