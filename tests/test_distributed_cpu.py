"""Multi-GPU layout on CPU ranks: poses are independent, the map is replicated, so N ranks each
simulate a contiguous pose shard and the concatenation must equal the single-process result.
Two gloo ranks on 127.0.0.1 run the oracle on their shards; no collective touches the data
path except the test's own gather."""
import os

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from rmagine_gb300 import scenes, sensors
from rmagine_gb300.simulation import pose_shard

IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)


def _rank(rank, world, port, out_q):
    import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc = scenes.box_room(seed=0, n_boxes=50)
    poses = scenes.room_poses(11, seed=1)
    lo, hi = pose_shard(poses.shape[0], rank, world)
    res = oracle.Scene(sc.vertices, sc.faces).simulate(sensors.vlp16_360(), IDENT, poses[lo:hi],
                                                       attrs=("ranges",), nthreads=1)["ranges"]
    parts = [None] * world
    dist.all_gather_object(parts, (lo, hi, res))
    if rank == 0:
        out_q.put(parts)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_pose_sharding_matches_single_process():
    import oracle

    world, port = 2, 29500 + (os.getpid() % 1000)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    parts = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sc = scenes.box_room(seed=0, n_boxes=50)
    poses = scenes.room_poses(11, seed=1)
    whole = oracle.Scene(sc.vertices, sc.faces).simulate(sensors.vlp16_360(), IDENT, poses, attrs=("ranges",))["ranges"]
    parts.sort(key=lambda x: x[0])
    assert parts[0][0] == 0 and parts[-1][1] == poses.shape[0]
    assert np.array_equal(np.concatenate([p[2] for p in parts]), whole)


def test_pose_shard_covers_all_poses_once():
    for n in (0, 1, 7, 100, 1001):
        for world in (1, 2, 3, 8):
            got = [pose_shard(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            assert max(h - l for l, h in got) - min(h - l for l, h in got) <= 1
