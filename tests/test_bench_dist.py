"""The replica path of bench.py on CPU: two gloo ranks, the max / sum helpers the timed
region uses (max over ranks of the step time, the whole-job sum of solves), and the
per-rank batch seeds (replicas solve different instances)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench
    w, r, local, dist = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank) and dist is not None
    mx = bench.dist_max(dist, 10.0 + rank)
    sm = bench.dist_sum(dist, 1.0 + rank)
    bench.dist_barrier(dist)
    meshes = bench.batch_meshes(2, seed=3 + 1000 * r)
    out[rank] = (mx, sm, meshes[0].m, meshes[0].name)
    dist.destroy_process_group()


def test_two_gloo_ranks():
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 11.0        # max over ranks
    assert res[0][1] == res[1][1] == 3.0         # whole-job sum
    assert res[0][3] != res[1][3] or res[0][2] != res[1][2]  # replicas solve different instances
