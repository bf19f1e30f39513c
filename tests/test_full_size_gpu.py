"""The full-size ray-casting workloads (1M- and 2.1M-triangle terrains with 2,000 boxes, 1,000 poses
of a 128 x 1024 spherical sensor or a 640 x 480 camera: 131 M and 307 M rays, all five attributes),
checked through properties that hold at any size:
* every walk (per ray, warp packet, 4-wide) and both tree builders give the same bytes -- the
  closest hit does not depend on the tree or the visiting order;
* two launches over the two halves of the poses give the bytes of one launch;
* the host-buffer entry point gives the bytes of the device form;
* a seeded sample of 20,000 rays agrees with the oracle (disputed rays certified in binary64);
* the attributes agree with one another: a hit has its range in [range.min, range.max] when flagged,
  its point is direction x range, its normal is unit length and faces the sensor; a miss writes
  range.max + 1, NaN points and normals and UINT32_MAX ids."""
import numpy as np
import pytest
import torch

import bench
import oracle
import rmagine_gb300 as rm

pytestmark = pytest.mark.gpu
IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)
MISS = 0xFFFFFFFF


@pytest.fixture(scope="module", autouse=True)
def _dev(built):
    torch.cuda.set_device(0)


def _simulate(sim, poses_dev, n, W, H, cfg=None):
    if cfg is not None:
        sim.launch_config = rm.launch_config(**cfg)
    b = rm.resize_memory_bundle(rm.Bundle(*bench.ALL), W, H, n, device="cuda")
    sim.simulate(poses_dev, b)
    torch.cuda.synchronize()
    return b


def _same(a, b, what):
    for k in bench.ALL:
        x, y = getattr(a, k), getattr(b, k)
        assert torch.equal(x.contiguous().view(torch.uint8), y.contiguous().view(torch.uint8)), (what, k)


def _consistent(b, model, dirs, W, H):
    rmin, rmax = np.float32(model.range.min), np.float32(model.range.max)
    r = b.ranges
    f = b.face_ids.view(torch.int32)
    hit = f != -1
    assert hit.float().mean() > 0.2
    assert torch.equal(b.hits.bool(), hit & (r >= float(rmin)))
    assert bool((r[hit] > 0).all()) and bool((r[hit] <= float(rmax)).all())
    assert bool((r[~hit] == float(np.float32(rmax + np.float32(1)))).all())
    pts, nrm = b.points.view(-1, 3), b.normals.view(-1, 3)
    assert bool(torch.isnan(pts[~hit]).all()) and bool(torch.isnan(nrm[~hit]).all())
    d = torch.from_numpy(dirs).cuda().repeat(r.numel() // (W * H), 1)
    want = d[hit] * r[hit, None]
    assert torch.equal(pts[hit], want)                       # points = dir_s * t, binary32
    nh = nrm[hit]
    assert float((nh.norm(dim=1) - 1).abs().max()) < 1e-5
    assert bool(((nh * d[hit]).sum(dim=1) <= 1e-6).all())   # faces the sensor


def _oracle_sample(sc, model, poses, b, n_rays, seed=0, k=20000):
    rng = np.random.default_rng(seed)
    gids = np.sort(rng.choice(n_rays, k, replace=False)).astype(np.uint64)
    scene = oracle.Scene(sc.vertices, sc.faces)
    o, d = scene.rays(model, IDENT, poses, gids)
    t, f = scene.trace_rays(o, d, float(model.range.max))
    rmin, rmax = np.float32(model.range.min), np.float32(model.range.max)
    want = {"face_ids": f, "ranges": np.where(f != MISS, t, rmax + np.float32(1)).astype(np.float32)}
    want["hits"] = ((f != MISS) & (want["ranges"] >= rmin)).astype(np.uint8)
    idx = torch.from_numpy(gids.astype(np.int64)).cuda()
    got = {"face_ids": b.face_ids.view(torch.int32)[idx].cpu().numpy().view(np.uint32),
           "ranges": b.ranges[idx].cpu().numpy(), "hits": b.hits[idx].cpu().numpy()}
    rep = oracle.certify(scene, model, IDENT, poses, got, want, gids=gids)
    assert rep["unexcused"] == 0, rep
    assert (got["face_ids"] != MISS).mean() > 0.2


@pytest.mark.parametrize("name", ["terrain1m_spherical", "terrain1m_pinhole", "terrain2m_spherical"])
def test_full_size_workload(name):
    sc, model, poses, attrs, _ = bench.raycast_workload(name)
    W, H = oracle.model_size(model)
    n = poses.shape[0]
    n_rays = n * W * H
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.make_simulator(model, m)
    P = torch.from_numpy(poses).cuda()
    ref = _simulate(sim, P, n, W, H, dict(packet=0, bvh_width=2))
    _consistent(ref, model, oracle.directions(model), W, H)
    _oracle_sample(sc, model, poses, ref, n_rays)
    m.build_wide8()
    for cfg in (dict(packet=1), dict(bvh_width=4, packet=0), dict(bvh_width=8, packet=0)):
        b = _simulate(sim, P, n, W, H, cfg)
        _same(ref, b, cfg)
        del b
    # two launches over the halves of the poses
    sim.launch_config = rm.launch_config(packet=0, bvh_width=2)
    halves = rm.resize_memory_bundle(rm.Bundle(*bench.ALL), W, H, n, device="cuda")
    for lo, hi in ((0, n // 2), (n // 2, n)):
        part = rm.Bundle(*bench.ALL)
        for k in bench.ALL:
            full = getattr(halves, k)
            per = full.shape[0] // n
            setattr(part, k, full[lo * per:hi * per])
        sim.simulate(P[lo:hi], part)
    torch.cuda.synchronize()
    _same(ref, halves, "halves")
    del halves
    # the LBVH of the same mesh
    lb = rm.make_simulator(model, rm.Map(sc.vertices, sc.faces, builder="lbvh"))
    b = _simulate(lb, P, n, W, H)
    _same(ref, b, "lbvh")
    del b, lb
    # the host-buffer entry point
    hb = rm.resize_memory_bundle(rm.Bundle(*bench.ALL), W, H, n, device="cpu", pin_memory=True)
    sim.simulate(torch.from_numpy(poses), hb)
    for k in bench.ALL:
        assert torch.equal(getattr(hb, k).view(torch.uint8), getattr(ref, k).cpu().view(torch.uint8)), ("host", k)
    assert m.status() == 0


def test_full_size_pose_gradient():
    """4,096 poses of a 64 x 1024 sensor on the 2.1M-triangle terrain (268 M rays): the fused forward
    equals plain simulate, each half of the poses gives the same rows, the host form gives the device
    result, the true poses give zero loss and gradient, and four sampled poses match the binary64
    analytic gradient of the oracle's ray set."""
    from test_pose_grad import rayset

    from rmagine_gb300 import grad as rg

    sc, model, true, est = bench.posegrad_workload(4096)
    W, H = oracle.model_size(model)
    n = true.shape[0]
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.SphereSimulator(m)
    sim.setModel(model)
    obs = sim.simulate(torch.from_numpy(true).cuda(), attrs=("ranges",)).ranges
    E = torch.from_numpy(est).cuda()
    g, loss, rs, fs = rg.range_pose_grad(sim, E, obs, 0.2, want_sim=True)
    plain = sim.simulate(E, attrs=("ranges", "face_ids"))
    torch.cuda.synchronize()
    assert torch.equal(plain.ranges, rs) and torch.equal(plain.face_ids, fs)
    assert float(loss.sum()) > 0
    half = n // 2
    for lo, hi in ((0, half), (half, n)):
        gh, lh = rg.range_pose_grad(sim, E[lo:hi], obs[lo * W * H:hi * W * H], 0.2)
        assert torch.equal(gh, g[lo:hi]) and torch.equal(lh, loss[lo:hi])
    gh, lh = rg.range_pose_grad(sim, torch.from_numpy(est).pin_memory(), obs.cpu().pin_memory(), 0.2)
    assert torch.equal(gh, g.cpu()) and torch.equal(lh, loss.cpu())
    g0, l0 = rg.range_pose_grad(sim, torch.from_numpy(true).cuda(), obs, 0.2)
    assert float(g0.abs().max()) == 0.0 and float(l0.abs().max()) == 0.0
    pick = np.array([0, 1234, 2900, 4095])
    sl = np.concatenate([np.arange(p * W * H, (p + 1) * W * H) for p in pick])
    rset, nn = rayset(sc, model, est[pick], fs.cpu().numpy().view(np.uint32)[sl], rs.cpu().numpy()[sl],
                      obs.cpu().numpy()[sl])
    an, an_loss = rset.analytic(nn, 0.2)
    got = g.cpu().numpy()[pick]
    assert np.abs(got - an).max() / np.abs(an).max() < 1e-3
    assert m.status() == 0


def test_full_size_fused_correction_step():
    """The fused simulate -> statistics_p2l -> Umeyama step for 1,000 estimates on the 1M-triangle
    terrain (131 M rays): each half of the estimates gives the same rows, the host form gives the
    device result, and at the true poses the correction is the identity."""
    from rmagine_gb300 import statistics as rs_

    sc, model, true, est = bench.rcc_workload(1000)
    W, H = oracle.model_size(model)
    n = true.shape[0]
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.SphereSimulator(m)
    sim.setModel(model)
    data = sim.simulate(torch.from_numpy(true).cuda(), attrs=("hits", "points"))
    dp, dm = data.points.reshape(n, W * H, 3), data.hits.reshape(n, W * H)
    P = rs_.UmeyamaReductionConstraints(max_dist=0.5)
    E = torch.from_numpy(est).cuda()
    st, T = sim.simulate_statistics(E, dp, dataset_mask=dm, params=P)
    torch.cuda.synchronize()
    counts = rs_.decode_stats(st)["n"]
    assert (counts > 0).mean() > 0.99 and counts.mean() > 1000, (int((counts == 0).sum()), float(counts.mean()))
    half = n // 2
    for lo, hi in ((0, half), (half, n)):
        sh, Th = sim.simulate_statistics(E[lo:hi], dp[lo:hi], dataset_mask=dm[lo:hi], params=P)
        assert torch.equal(sh, st[lo:hi]) and torch.equal(Th, T[lo:hi])
    sh, Th = sim.simulate_statistics(torch.from_numpy(est), dp.cpu(), dataset_mask=dm.cpu(), params=P)
    assert torch.equal(sh.cpu(), st.cpu()) and torch.equal(Th.cpu(), T.cpu())
    _, T0 = sim.simulate_statistics(torch.from_numpy(true).cuda(), dp, dataset_mask=dm, params=P)
    T0 = T0.cpu().numpy()
    assert np.abs(T0[:, :3]).max() < 1e-5 and np.abs(np.abs(T0[:, 3]) - 1).max() < 1e-6
    assert np.abs(T0[:, 4:7]).max() < 1e-4
    assert m.status() == 0


def test_full_size_batched_sensors():
    """The 64-sensor mix of the batched benchmark (9.0 G rays on the 2.1M-triangle terrain,
    Hits + Ranges): one batched launch gives every sensor the bytes of its own plain launch."""
    from rmagine_gb300 import batched, scenes

    sc = scenes.terrain(grid=1024, n_boxes=2000, seed=0)
    m = rm.Map(sc.vertices, sc.faces)
    spec = batched.mixed_sensor_set(64, seed=0)
    attrs = ("hits", "ranges")
    jobs, total = [], 0
    for i, (mod, c) in enumerate(spec):
        sim = rm.make_simulator(mod, m)
        poses = torch.from_numpy(scenes.terrain_poses(sc, c, seed=100 + i)).cuda()
        b = rm.resize_memory_bundle(rm.Bundle(*attrs), sim.sensor.width, sim.sensor.height, c, device="cuda")
        jobs.append((sim, poses, b))
        total += sim.sensor.width * sim.sensor.height * c
    assert total > 8e9
    plan = batched.BatchPlan(m, jobs)
    plan.launch()
    torch.cuda.synchronize()
    for sim, poses, b in jobs:
        p = sim.simulate(poses, attrs=attrs)
        for a in attrs:
            assert torch.equal(getattr(b, a).view(torch.uint8), getattr(p, a).view(torch.uint8)), a
        del p
    assert m.status() == 0


def test_full_size_instanced_scene():
    """The instanced benchmark scene (1M-triangle terrain with its tree opened into pieces + 2,000
    box instances, 1,000 poses, 131 M rays, all seven attributes): two launches over the halves of the
    poses give the bytes of one, the host form the device result, and a seeded sample of 20,000 rays
    matches the scene oracle (which tries every instance whole)."""
    from oracle.scene import InstancedScene
    from rmagine_gb300 import scenes, sensors

    meshes, insts, baked = scenes.instanced_terrain(grid=708, n_boxes=2000, seed=0)
    model = sensors.ouster_like(128, 1024, 45.0, 0.5, 130.0)
    poses = scenes.terrain_poses(baked, 1000, seed=2)
    W, H = oracle.model_size(model)
    n = poses.shape[0]
    geoms = [rm.Map(v, f) for v, f in meshes]
    scene = rm.Scene(geoms, [rm.Instance(i["geometry"], i["T"], i["scale"], i["geom_id"], i["object_id"])
                             for i in insts])
    sim = rm.make_simulator(model, scene)
    A = rm.ATTRIBUTES
    P = torch.from_numpy(poses).cuda()
    ref = rm.resize_memory_bundle(rm.Bundle(*A), W, H, n, device="cuda")
    sim.simulate(P, ref)
    halves = rm.resize_memory_bundle(rm.Bundle(*A), W, H, n, device="cuda")
    for lo, hi in ((0, n // 2), (n // 2, n)):
        part = rm.Bundle(*A)
        for k in A:
            full = getattr(halves, k)
            per = full.shape[0] // n
            setattr(part, k, full[lo * per:hi * per])
        sim.simulate(P[lo:hi], part)
    torch.cuda.synchronize()
    for k in A:
        assert torch.equal(getattr(ref, k).view(torch.uint8), getattr(halves, k).view(torch.uint8)), k
    del halves
    hb = rm.resize_memory_bundle(rm.Bundle(*A), W, H, n, device="cpu", pin_memory=True)
    sim.simulate(torch.from_numpy(poses), hb)
    for k in A:
        assert torch.equal(getattr(hb, k).view(torch.uint8), getattr(ref, k).cpu().view(torch.uint8)), ("host", k)
    # oracle on a sample of rays: every instance tried whole, disputed rays certified in binary64
    rng = np.random.default_rng(5)
    gids = np.sort(rng.choice(n * W * H, 20000, replace=False)).astype(np.uint64)
    osc = InstancedScene(meshes, insts)
    o, d = osc._ray_scene.rays(model, IDENT, poses, gids)
    t, inst, f = osc.trace(o, d, float(model.range.max))
    rmin, rmax = np.float32(model.range.min), np.float32(model.range.max)
    obj = np.array([I["object_id"] for I in osc.instances], np.uint32)
    want = {"face_ids": f, "ranges": np.where(f != MISS, t, rmax + np.float32(1)).astype(np.float32),
            "object_ids": np.where(inst >= 0, obj[np.maximum(inst, 0)], MISS).astype(np.uint32)}
    idx = torch.from_numpy(gids.astype(np.int64)).cuda()
    got = {"face_ids": ref.face_ids[idx].cpu().numpy().view(np.uint32), "ranges": ref.ranges[idx].cpu().numpy(),
           "object_ids": ref.object_ids[idx].cpu().numpy().view(np.uint32)}
    rep = osc.certify(model, IDENT, poses, got, want, gids=gids)
    assert rep["unexcused"] == 0, rep
    assert (got["face_ids"] != MISS).mean() > 0.2
    assert scene.status() == 0


def test_full_size_icp_statistics():
    """The ICP workload (8,192 batches x 32,768 correspondences, 6.4 GB of points): statistics,
    Umeyama and the backward of each half of the batches give the rows of one call, and four sampled
    batches match the binary64 two-pass statistics of the oracle."""
    from oracle import stats as ost

    from rmagine_gb300 import statistics as rs_

    src, tgt = bench.icp_data(8192, 32768, torch.device("cuda", 0))
    B = src.shape[0]
    st, T = rs_.statistics(src, tgt)
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    gR = torch.randn((B, 9), generator=g, device="cuda")
    gt = torch.randn((B, 3), generator=g, device="cuda")
    gd, gm = rs_.umeyama_backward(src, tgt, st, gR, gt)
    torch.cuda.synchronize()
    h = B // 2
    for lo, hi in ((0, h), (h, B)):
        sh, Th = rs_.statistics(src[lo:hi], tgt[lo:hi])
        assert torch.equal(sh, st[lo:hi]) and torch.equal(Th, T[lo:hi])
        dh, mh = rs_.umeyama_backward(src[lo:hi], tgt[lo:hi], sh, gR[lo:hi], gt[lo:hi])
        assert torch.equal(dh, gd[lo:hi]) and torch.equal(mh, gm[lo:hi])
    pick = [0, 2047, 5000, 8191]
    got = rs_.decode_stats(st[pick])
    want = ost.stats(*ost.correspondences(src[pick].cpu().numpy(), tgt[pick].cpu().numpy()))
    assert np.array_equal(got["n"], want["n"])
    assert np.abs(got["dataset_mean"] - want["dataset_mean"]).max() <= 2e-5 * (1 + np.abs(want["dataset_mean"]).max())
    assert np.abs(got["model_mean"] - want["model_mean"]).max() <= 2e-5 * (1 + np.abs(want["model_mean"]).max())
    scale = np.abs(want["covariance"]).max(axis=(1, 2), keepdims=True)
    assert (np.abs(got["covariance"] - want["covariance"]) / scale).max() <= 2e-6
    assert bool(torch.isfinite(gd).all()) and bool(torch.isfinite(gm).all())
