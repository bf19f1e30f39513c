"""Batched heterogeneous sensors: one persistent graph-replayed launch must reproduce one plain
rmg_simulate per sensor bit for bit, for every launch option the autotuner can pick."""
import numpy as np
import pytest
import torch

import rmagine_gb300 as rm
from rmagine_gb300 import batched, scenes, sensors

pytestmark = pytest.mark.gpu
ATTRS = ("hits", "ranges", "normals", "face_ids")
IDENT_T = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)


@pytest.fixture(scope="module")
def setup(built):
    torch.cuda.set_device(0)
    sc = scenes.terrain(grid=128, n_boxes=200, seed=40)
    m = rm.Map(sc.vertices, sc.faces)
    rng = np.random.default_rng(41)
    models = [sensors.vlp16_900(), sensors.ouster_like(32, 256), sensors.depth_camera(64, 48),
              sensors.O1DnModel(width=777, height=1, range=sensors.Interval(0.3, 130.0), orig=(0.1, 0.0, 0.2),
                                dirs=sensors.sphere_directions(777, seed=42)),
              sensors.OnDnModel(width=33, height=5, range=sensors.Interval(0.0, 130.0),
                                origs=rng.uniform(-0.3, 0.3, (165, 3)).astype(np.float32),
                                dirs=sensors.sphere_directions(165, seed=43)),
              sensors.ouster_like(16, 100)]
    counts = [1, 7, 3, 12, 2, 5]
    jobs, plains = [], []
    for i, (mod, c) in enumerate(zip(models, counts)):
        sim = rm.make_simulator(mod, m)
        if i == 3:
            sim.setTsb(np.array([0, 0, np.sin(0.1), np.cos(0.1), 0.2, 0.0, 0.1, 0], np.float32))
        poses = torch.from_numpy(scenes.terrain_poses(sc, c, seed=50 + i)).cuda()
        b = rm.resize_memory_bundle(rm.Bundle(*ATTRS), sim.sensor.width, sim.sensor.height, c, device="cuda")
        jobs.append((sim, poses, b))
        plains.append(sim.simulate(poses, attrs=ATTRS))
    torch.cuda.synchronize()
    return m, jobs, plains


def assert_same(jobs, plains):
    for (sim, poses, b), p in zip(jobs, plains):
        for a in ATTRS:
            x, y = getattr(b, a), getattr(p, a)
            assert torch.equal(x.view(torch.uint8), y.view(torch.uint8)), a


def clear(jobs):
    for _, _, b in jobs:
        for t in b.tensors().values():
            t.fill_(0x55) if t.dtype == torch.uint8 else t.view(torch.int32).fill_(0x5555)


@pytest.mark.parametrize("cfg", [dict(), dict(stack_depth=0, block_warps=2, grab=1),
                                 dict(stack_depth=16, block_warps=8, tile_w=4, tile_h=8, grab=4),
                                 dict(use_graph=0, tile_w=16, tile_h=2), dict(ctas_per_sm=1, grab=7)])
def test_batched_equals_plain(setup, cfg):
    m, jobs, plains = setup
    plan = batched.BatchPlan(m, jobs, batched.batch_config(**cfg))
    for _ in range(2):  # replaying the graph twice gives the same result
        clear(jobs)
        plan.launch()
        torch.cuda.synchronize()
        assert_same(jobs, plains)
    assert m.status() == 0
    info = plan.info()
    assert info["rays"] == sum(s.sensor.width * s.sensor.height * p.shape[0] for s, p, _ in jobs)


def test_autotune_picks_a_valid_config_and_keeps_results(setup, tmp_path):
    m, jobs, plains = setup
    plan = batched.BatchPlan(m, jobs)
    best = plan.autotune(reps=2, cache=tmp_path / "tune.json")
    assert best.stack_depth in (0, 8, 16) and 1 <= best.block_warps <= 8 and best.tile_w * best.tile_h == 32
    clear(jobs)
    plan.launch()
    torch.cuda.synchronize()
    assert_same(jobs, plains)
    # the cached choice is reused by a second plan with the same signature
    plan2 = batched.BatchPlan(m, jobs)
    again = plan2.autotune(reps=2, cache=tmp_path / "tune.json")
    assert [again.stack_depth, again.block_warps, again.tile_w, again.grab] == \
        [best.stack_depth, best.block_warps, best.tile_w, best.grab]


def test_empty_plan_and_zero_pose_entries(setup):
    m, jobs, plains = setup
    plan = batched.BatchPlan(m, [])
    plan.launch()
    torch.cuda.synchronize()
    assert plan.info()["rays"] == 0


@pytest.mark.parametrize("n_chunks", [1, 3, 8])
def test_chunked_plan_to_host_equals_plain(setup, n_chunks):
    """ChunkedBatchPlan.run_to_host: every job's poses in n_chunks ranges (jobs with fewer poses sit
    in the first ranges), outputs copied to pinned and pageable host bundles bit-identical to one
    plain simulate per sensor; launch() alone fills the device bundles the same way."""
    m, jobs, plains = setup
    cp = batched.ChunkedBatchPlan(m, jobs, n_chunks)
    for pin in (True, False):
        hosts = []
        for sim, poses, b in jobs:
            hb = rm.resize_memory_bundle(rm.Bundle(*ATTRS), sim.sensor.width, sim.sensor.height, poses.shape[0],
                                         device="cpu", pin_memory=pin)
            for t in hb.tensors().values():
                t.view(torch.uint8).fill_(0xA5)
            hosts.append(hb)
        clear(jobs)
        cp.run_to_host(hosts)
        for hb, p in zip(hosts, plains):
            for a in ATTRS:
                assert torch.equal(getattr(hb, a).view(torch.uint8), getattr(p, a).cpu().view(torch.uint8)), a
    clear(jobs)
    cp.launch()
    torch.cuda.synchronize()
    assert_same(jobs, plains)
    assert m.status() == 0


def test_batched_mixed_sensors_match_the_oracle(built):
    """One batched launch over all four sensor kinds with ragged pose counts (1 to 9 poses, a sensor
    offset on one of them), checked against the oracle's restatement of the Embree path directly --
    not only against plain launches -- with the binary64 certifier for disputed rays."""
    import oracle

    torch.cuda.set_device(0)
    sc = scenes.terrain(grid=96, n_boxes=120, seed=60)
    m = rm.Map(sc.vertices, sc.faces)
    rng = np.random.default_rng(61)
    models = [sensors.ouster_like(16, 128), sensors.depth_camera(48, 36),
              sensors.O1DnModel(width=500, height=1, range=sensors.Interval(0.3, 130.0), orig=(0.1, 0.0, 0.2),
                                dirs=sensors.sphere_directions(500, seed=62)),
              sensors.OnDnModel(width=25, height=8, range=sensors.Interval(0.0, 130.0),
                                origs=rng.uniform(-0.3, 0.3, (200, 3)).astype(np.float32),
                                dirs=sensors.sphere_directions(200, seed=63)),
              sensors.vlp16_900()]
    counts = [9, 1, 4, 7, 2]
    tsbs = [IDENT_T, IDENT_T, np.array([0, 0, np.sin(0.1), np.cos(0.1), 0.2, 0.0, 0.1, 0], np.float32), IDENT_T,
            IDENT_T]
    attrs = ("hits", "ranges", "face_ids")
    jobs = []
    for i, (mod, c, tsb) in enumerate(zip(models, counts, tsbs)):
        sim = rm.make_simulator(mod, m)
        sim.setTsb(tsb)
        poses = torch.from_numpy(scenes.terrain_poses(sc, c, seed=70 + i)).cuda()
        b = rm.resize_memory_bundle(rm.Bundle(*attrs), sim.sensor.width, sim.sensor.height, c, device="cuda")
        jobs.append((sim, poses, b))
    plan = batched.BatchPlan(m, jobs)
    plan.launch()
    torch.cuda.synchronize()
    assert m.status() == 0
    osc = oracle.Scene(sc.vertices, sc.faces)
    for (sim, poses, b), mod, tsb in zip(jobs, models, tsbs):
        got = {"hits": b.hits.cpu().numpy(), "ranges": b.ranges.cpu().numpy(),
               "face_ids": b.face_ids.cpu().numpy().view(np.uint32)}
        Tbm = poses.cpu().numpy()
        want = osc.simulate(mod, tsb, Tbm, attrs=attrs)
        rep = oracle.certify(osc, mod, tsb, Tbm, got, want)
        assert rep["unexcused"] == 0, rep
        assert rep["disputed"] <= 1e-3 * rep["rays"], rep
        agree = got["face_ids"] == want["face_ids"]
        assert np.array_equal(got["hits"][agree], want["hits"][agree])
        assert np.array_equal(got["ranges"][agree].view(np.uint32), want["ranges"][agree].view(np.uint32))
