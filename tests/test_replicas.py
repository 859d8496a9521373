"""bench.py --gpus N runs N independent replicas (the shooting loop is strictly
sequential, so there is nothing to shard): the only collectives are the
barrier and the max over ranks.  Exercised here with gloo, world size 2, CPU."""
import os
import socket

import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, REPO)
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import bench
    w, r, l = bench.rank_env()
    ranks = bench.Ranks(w, "gloo")
    ranks.barrier()
    my_ms = 100.0 + 50.0 * r              # rank 1 is the slow one
    worst = ranks.max(my_ms)
    out[r] = (worst, bench.replica_value(w, 40, worst))
    ranks.barrier()
    ranks.close()


def test_replicas_max_over_ranks_gloo():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    assert out[0] == out[1]
    worst, value = out[0]
    assert worst == 150.0
    assert abs(value - 2 * 40 / 0.150) < 1e-9


def test_single_rank_has_no_collective():
    import sys
    sys.path.insert(0, REPO)
    import bench
    r = bench.Ranks(1, "gloo")
    assert r.dist is None and r.max(3.5) == 3.5
