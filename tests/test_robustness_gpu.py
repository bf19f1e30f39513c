"""Geometry that breaks careless ray casters, on the GPU against the oracle:
* watertightness: from inside a closed mesh every ray hits, including rays aimed exactly at shared
  vertices and edges (the watertight triangle test has no gaps between neighbours);
* degenerate and sliver triangles mixed into a scene;
* a scene 10 km from the coordinate origin.
Both tree builders and every walk give bit-identical results."""
import numpy as np
import pytest
import torch

import oracle
import rmagine_gb300 as rm
from meshes import icosphere
from rmagine_gb300 import scenes, sensors

pytestmark = pytest.mark.gpu
IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)
WALKS = [dict(packet=0), dict(packet=1), dict(bvh_width=4, packet=0), dict(bvh_width=8, packet=0),
         dict(stack_depth=0, packet=0)]


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    torch.cuda.set_device(0)


def run(m, model, poses, cfg=None, attrs=rm.ATTRIBUTES):
    sim = rm.make_simulator(model, m)
    if cfg is not None:
        sim.launch_config = rm.launch_config(**cfg)
    res = sim.simulate(torch.from_numpy(np.ascontiguousarray(poses, np.float32)).cuda(), attrs=attrs)
    torch.cuda.synchronize()
    out = {}
    for a in attrs:
        t = getattr(res, a).cpu().numpy()
        out[a] = t.view(np.uint32) if a.endswith("_ids") else t
    return out


def same(a, b):
    return all(np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)) for k in a)


def check_everything(v, f, model, poses):
    """Parity with the oracle (certified) on the SAH map, and bit-identical results on the LBVH map
    and for every walk."""
    sah, lbvh = rm.Map(v, f).build_wide8(), rm.Map(v, f, builder="lbvh").build_wide8()
    got = run(sah, model, poses)
    sc = oracle.Scene(v, f)
    want = sc.simulate(model, IDENT, poses)
    rep = oracle.certify(sc, model, IDENT, poses, got, want)
    assert rep["unexcused"] == 0, rep
    for m in (sah, lbvh):
        for cfg in WALKS:
            assert same(run(m, model, poses, cfg), got), cfg
        assert m.status() == 0
    return got


def test_closed_sphere_has_no_gaps_at_shared_vertices_and_edges():
    v, f = icosphere(3, radius=2.0)                   # 1,280 triangles, 642 vertices, 1,920 edges
    edges = {(min(a, b), max(a, b)) for tri in f for a, b in ((tri[0], tri[1]), (tri[1], tri[2]), (tri[2], tri[0]))}
    targets = np.concatenate([v.astype(np.float64),
                              np.array([(v[a].astype(np.float64) + v[b]) / 2 for a, b in sorted(edges)])])
    rng = np.random.default_rng(3)
    targets = np.concatenate([targets, rng.standard_normal((2000, 3))])
    for centre in (np.zeros(3), np.array([0.31, -0.17, 0.05])):
        dirs = targets - centre
        dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
        model = sensors.O1DnModel(width=dirs.shape[0], height=1, range=sensors.Interval(0.0, 10.0),
                                  orig=(0.0, 0.0, 0.0), dirs=dirs)
        pose = IDENT.copy()
        pose[4:7] = centre
        got = check_everything(v, f, model, pose[None])
        assert np.all(got["hits"] == 1), int((got["hits"] == 0).sum())
        assert np.all(got["face_ids"] != 0xFFFFFFFF)


def test_degenerate_and_sliver_triangles():
    room = scenes.box_room(seed=71, n_boxes=60)
    rng = np.random.default_rng(72)
    vs, fs = [room.vertices], [room.faces]
    base = room.vertices.shape[0]
    extra_v, extra_f = [], []
    for i in range(300):
        p = rng.uniform([-9, -9, 0.2], [9, 9, 3.5]).astype(np.float32)
        kind = i % 3
        if kind == 0:    # all three vertices equal
            tri = np.stack([p, p, p])
        elif kind == 1:  # collinear
            d = rng.standard_normal(3).astype(np.float32)
            tri = np.stack([p, p + d, p + 2 * d])
        else:            # sliver: 1e-6 m wide, 2 m long
            d = rng.standard_normal(3).astype(np.float32)
            tri = np.stack([p, p + d, p + d + np.float32(1e-6)])
        extra_v.append(tri)
        extra_f.append(base + 3 * i + np.arange(3))
    v = np.concatenate(vs + extra_v).astype(np.float32)
    f = np.concatenate(fs + [np.array(extra_f, np.uint32)]).astype(np.uint32)
    check_everything(v, f, sensors.vlp16_900(), scenes.room_poses(6, seed=73))


def test_scene_ten_km_from_the_origin():
    room = scenes.box_room(seed=74, n_boxes=80)
    off = np.array([1.0e4, -7.5e3, 120.0])
    v = (room.vertices.astype(np.float64) + off).astype(np.float32)
    poses = scenes.room_poses(6, seed=75)
    poses[:, 4:7] += off.astype(np.float32)
    check_everything(v, room.faces, sensors.vlp16_900(), poses)
