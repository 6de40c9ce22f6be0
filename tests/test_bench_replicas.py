"""The multi-GPU path of bench.py is replicas only: each rank runs the whole
workload, the ranks meet at barriers around the timed region and the job's
time is the maximum over ranks.  Exercised here with two gloo ranks on CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(REPO))
    import bench
    r, w, local, dist = bench.dist_setup(world)
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, 10.0 + 5.0 * r)      # rank 1 is the slower replica
    out[r] = (r, w, local, t, bench.replica_mlups(w, 1000, 4, t))
    bench.barrier(dist)
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for r in (0, 1):
        rank, world, local, t, mlups = res[r]
        assert (rank, world, local) == (r, 2, r)
        assert t == 15.0                                  # max over ranks
        assert mlups == pytest.approx(2 * 1000 * 4 / 15e-3 / 1e6)
