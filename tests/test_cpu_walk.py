"""The timed CPU baseline's walk (the oracle's Embree-style 4-wide SIMD walk, orc_simulate4)
gives the same outputs as the oracle's restatement, bit for bit, on every workload kind and on
the geometry that breaks careless ray casters: closed meshes hit at shared vertices and edges,
axis-parallel rays lying in box faces, degenerate and sliver triangles, a scene 10 km from the
origin, one-leaf and empty trees."""
import numpy as np
import pytest

import oracle
from meshes import icosphere
from rmagine_gb300 import scenes, sensors

IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)


def both(v, f, model, poses, max_leaf=4, attrs=("hits", "ranges", "points", "normals", "face_ids")):
    sc = oracle.Scene(v, f, max_leaf=max_leaf)
    want = sc.simulate(model, IDENT, poses, attrs=attrs)
    got = sc.simulate(model, IDENT, poses, attrs=attrs, fast=True)
    for a in attrs:
        assert np.array_equal(want[a].view(np.uint8), got[a].view(np.uint8)), a
    return got


@pytest.mark.parametrize("max_leaf", [1, 4, 15])
def test_terrain_spherical(max_leaf):
    sc = scenes.terrain(grid=160, n_boxes=60, seed=5)
    got = both(sc.vertices, sc.faces, sensors.ouster_like(32, 256, 45.0, 0.5, 130.0),
               scenes.terrain_poses(sc, 3, seed=6), max_leaf=max_leaf)
    assert 0.2 < got["hits"].mean() < 1.0


def test_terrain_pinhole_and_room_vlp16():
    sc = scenes.terrain(grid=120, n_boxes=40, seed=7)
    both(sc.vertices, sc.faces, sensors.depth_camera(64, 48, 90.0, 0.3, 130.0), scenes.terrain_poses(sc, 3, seed=8))
    room = scenes.box_room(seed=9, n_boxes=80)
    got = both(room.vertices, room.faces, sensors.vlp16_900(), scenes.room_poses(4, seed=10))
    assert got["hits"].mean() > 0.5


def test_o1dn_ondn_examples():
    room = scenes.box_room(seed=11, n_boxes=30)
    for model in (sensors.example_o1dn(), sensors.example_ondn()):
        both(room.vertices, room.faces, model, scenes.room_poses(5, seed=12))


def test_closed_sphere_vertices_edges_and_axis_rays():
    v, f = icosphere(2, radius=2.0)
    edges = {(min(a, b), max(a, b)) for tri in f for a, b in ((tri[0], tri[1]), (tri[1], tri[2]), (tri[2], tri[0]))}
    axis = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                     [1, 1, 0], [0, -1, 1], [1, 0, -1]], np.float64)
    targets = np.concatenate([v.astype(np.float64), np.array([(v[a].astype(np.float64) + v[b]) / 2 for a, b in
                                                              sorted(edges)])])
    for centre in (np.zeros(3), np.array([0.31, -0.17, 0.05])):
        dirs = targets - centre
        dirs = np.concatenate([dirs / np.linalg.norm(dirs, axis=1, keepdims=True),
                               axis / np.linalg.norm(axis, axis=1, keepdims=True)]).astype(np.float32)
        model = sensors.O1DnModel(width=dirs.shape[0], height=1, range=sensors.Interval(0.0, 10.0),
                                  orig=(0.0, 0.0, 0.0), dirs=dirs)
        pose = IDENT.copy()
        pose[4:7] = centre
        got = both(v, f, model, pose[None], max_leaf=1)
        assert np.all(got["hits"] == 1)


def test_axis_parallel_rays_in_box_faces():
    # origins on the faces and edges of axis-aligned boxes, directions along the axes: the slab
    # tests meet planes they lie in (zero direction components, 1/d replaced by +-1e20)
    v, f = scenes.merge([scenes.box_mesh([-1, -1, -1], [1, 1, 1]), scenes.box_mesh([2, -1, -1], [3, 1, 1]),
                         scenes.box_mesh([-1, 2, -1], [1, 3, 0])])
    dirs = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    model = sensors.O1DnModel(width=dirs.shape[0], height=1, range=sensors.Interval(0.0, 50.0),
                              orig=(0.0, 0.0, 0.0), dirs=dirs)
    poses = []
    for o in ([1, 0, 0], [1, 1, 0], [1, 1, 1], [-1, 0.5, 0], [2, 0, 0], [0, 2, 0], [0, 3, -1], [1.5, 1, 1],
              [0, 0, 0], [2.5, -1, 1]):
        p = IDENT.copy()
        p[4:7] = o
        poses.append(p)
    for ml in (1, 4):
        both(v, f, model, np.array(poses), max_leaf=ml)


def test_degenerate_triangles_and_far_from_origin():
    room = scenes.box_room(seed=13, n_boxes=40)
    rng = np.random.default_rng(14)
    extra = []
    for i in range(120):
        p = rng.uniform([-9, -9, 0.2], [9, 9, 3.5]).astype(np.float32)
        d = rng.standard_normal(3).astype(np.float32)
        extra.append([np.stack([p, p, p]), np.stack([p, p + d, p + 2 * d]),
                      np.stack([p, p + d, p + d + np.float32(1e-6)])][i % 3])
    base = room.vertices.shape[0]
    v = np.concatenate([room.vertices] + extra).astype(np.float32)
    f = np.concatenate([room.faces, base + np.arange(3 * len(extra), dtype=np.uint32).reshape(-1, 3)])
    both(v, f, sensors.vlp16_900(), scenes.room_poses(3, seed=15))
    off = np.array([1.0e4, -7.5e3, 120.0])
    poses = scenes.room_poses(3, seed=16)
    poses[:, 4:7] += off.astype(np.float32)
    both((room.vertices.astype(np.float64) + off).astype(np.float32), room.faces, sensors.vlp16_900(), poses)


def test_one_leaf_and_empty_trees():
    model = sensors.vlp16_360()
    poses = scenes.room_poses(2, seed=17)
    v, f = scenes.box_mesh([-3, -3, -1], [3, 3, 3])
    for n in (1, 3, 4):  # the whole tree is one leaf of max_leaf = 4
        both(v, f[:n], model, poses)
    got = both(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32), model, poses)
    assert np.all(got["hits"] == 0) and np.all(got["face_ids"] == 0xFFFFFFFF)


def test_leaf_too_large_is_refused():
    v, f = scenes.box_mesh([-1, -1, -1], [1, 1, 1])
    vv = np.concatenate([v + np.float32(3 * i) for i in range(2)]).astype(np.float32)
    ff = np.concatenate([f, f + v.shape[0]]).astype(np.uint32)  # 24 triangles in one leaf
    sc = oracle.Scene(vv, ff, max_leaf=32)
    with pytest.raises(ValueError):
        sc.simulate(sensors.vlp16_360(), IDENT, IDENT[None], fast=True)
