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
    for cfg in (dict(packet=1), dict(bvh_width=4, packet=0)):
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
