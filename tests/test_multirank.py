"""The N > 1 path of bench.py on CPU: two gloo ranks (replicas; the Voronoi
path needs no data exchange), barrier and max-over-ranks timing."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import numpy as np

    import bench

    env = bench.dist_env()
    dist = bench.dist_init(env[0], "gloo")
    t = bench.max_over_ranks(dist, 1.0 + rank)
    bench.barrier(dist)
    # replicas: every rank generates the same workload from the same seed
    pts, _ = bench.make_points("uniform1m")
    q.put((env, t, float(np.sum(pts[:1000]))))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(r[0][1] for r in res) == [0, 1]
    assert all(r[0][0] == 2 for r in res)
    assert all(r[1] == 2.0 for r in res)            # max over ranks
    assert res[0][2] == res[1][2]
