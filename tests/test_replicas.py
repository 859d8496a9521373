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


def _shard_worker(rank, world, port, out):
    """Each rank takes its share of the 256-room batch (balanced by triangle
    count, no data exchanged); the shares are gathered only to check them."""
    import sys
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "hw-radiosity_gb300"))
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import torch.distributed as dist
    from hwrad import scenes, shard
    import bench
    w, r, _ = bench.rank_env()
    ranks = bench.Ranks(w, "gloo")
    tris = [len(g.vtx) for g in scenes.batch_rooms(256, seed=4000)]
    mine = shard.partition_scenes(tris, w)[r]
    shares = [None] * w
    dist.all_gather_object(shares, mine)
    total = ranks.sum(float(sum(tris[i] for i in mine)))
    out[r] = (shares, total, sum(tris[i] for i in mine))
    ranks.barrier()
    ranks.close()


def test_batch_scene_shards_cover_every_scene_once_gloo():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_shard_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    shares0, total0, load0 = out[0]
    shares1, total1, load1 = out[1]
    assert shares0 == shares1                       # every rank computed the same partition
    flat = sorted(i for s in shares0 for i in s)
    assert flat == list(range(256))                 # each scene exactly once
    assert total0 == total1 == load0 + load1        # the sum over ranks is the whole batch
    assert max(load0, load1) / min(load0, load1) < 1.01   # balanced by triangle count


def test_partition_scenes_edges():
    import sys
    sys.path.insert(0, os.path.join(REPO, "hw-radiosity_gb300"))
    from hwrad import shard
    assert shard.partition_scenes([], 3) == [[], [], []]
    assert shard.partition_scenes([5, 1, 1], 1) == [[0, 1, 2]]
    assert shard.partition_scenes([5, 1, 1, 1], 2) == [[0], [1, 2, 3]]
    parts = shard.partition_scenes([3, 3, 3], 5)
    assert sorted(i for p in parts for i in p) == [0, 1, 2] and sum(1 for p in parts if not p) == 2
