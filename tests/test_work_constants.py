"""The per-ray work constants bench.py uses for its roofline (mean LBVH node visits and triangle
tests per ray) re-derived by the oracle's instrumented traversal on smaller samples."""
import numpy as np
import pytest

import bench
import oracle

IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)


@pytest.mark.parametrize("name", ["terrain1m_spherical", "room_vlp16"])
def test_work_per_ray_constants(name):
    sc, model, poses, attrs, desc = bench.raycast_workload(name)
    W, H = oracle.model_size(model)
    n = poses.shape[0] * W * H
    rng = np.random.default_rng(1)
    gids = np.sort(rng.choice(n, min(n, 40000), replace=False)).astype(np.uint64)
    o, d = oracle.Scene(sc.vertices, sc.faces).rays(model, IDENT, poses, gids)
    v, t, _, _ = oracle.CanonicalLbvh(sc.vertices, sc.faces).count(o, d, model.range.max)
    want = bench.WORK_PER_RAY[name]
    assert abs(v.mean() - want["nodes"]) / want["nodes"] < 0.03
    assert abs(t.mean() - want["tris"]) / want["tris"] < 0.05


def test_rcc_fused_work_constants():
    """rcc_fused casts only rays whose dataset point is valid (a hit at the true pose); its
    constants average node visits / triangle tests at the estimates over all sensor rays."""
    sc, model, true, est = bench.rcc_workload(1000)
    W, H = oracle.model_size(model)
    n = true.shape[0] * W * H
    rng = np.random.default_rng(1)
    gids = np.sort(rng.choice(n, 40000, replace=False)).astype(np.uint64)
    scene = oracle.Scene(sc.vertices, sc.faces)
    lbvh = oracle.CanonicalLbvh(sc.vertices, sc.faces)
    o, d = scene.rays(model, IDENT, true, gids)
    _, _, t, f = lbvh.count(o, d, model.range.max)
    valid = (f != 0xFFFFFFFF) & (t >= model.range.min)
    o, d = scene.rays(model, IDENT, est, gids)
    v, tt, _, _ = lbvh.count(o, d, model.range.max)
    want = bench.WORK_PER_RAY["rcc_fused"]
    assert abs(valid.mean() - want["data_frac"]) < 0.01
    assert abs(np.where(valid, v, 0).mean() - want["nodes"]) / want["nodes"] < 0.03
    assert abs(np.where(valid, tt, 0).mean() - want["tris"]) / want["tris"] < 0.05


# SAH yardstick (oracle binned-SAH tree, one triangle per leaf, same visiting order and culling)
SAH_YARDSTICK = {"terrain1m_spherical": {"nodes": 25.206, "tris": 1.721}, "room_vlp16": {"nodes": 24.502, "tris": 3.124}}


@pytest.mark.parametrize("name", ["terrain1m_spherical", "room_vlp16"])
def test_sah_yardstick(name):
    """The tree-quality yardstick beside the LBVH constants: mean node visits and triangle tests per
    ray through the oracle's binned-SAH tree (one triangle per leaf) on the same rays, which must
    find the same closest faces as the LBVH."""
    sc, model, poses, attrs, desc = bench.raycast_workload(name)
    W, H = oracle.model_size(model)
    n = poses.shape[0] * W * H
    rng = np.random.default_rng(1)
    gids = np.sort(rng.choice(n, min(n, 40000), replace=False)).astype(np.uint64)
    o, d = oracle.Scene(sc.vertices, sc.faces).rays(model, IDENT, poses, gids)
    _, _, _, lf = oracle.CanonicalLbvh(sc.vertices, sc.faces).count(o, d, model.range.max)
    v, t, _, f = oracle.Scene(sc.vertices, sc.faces, max_leaf=1).count(o, d, model.range.max)
    assert np.array_equal(f, lf)
    want = SAH_YARDSTICK[name]
    assert abs(v.mean() - want["nodes"]) / want["nodes"] < 0.03
    assert abs(t.mean() - want["tris"]) / want["tris"] < 0.05


def test_tree_count_of_an_exported_tree_equals_the_canonical_walk():
    """oracle.tree_count (any tree in the GPU layout) walks like CanonicalLbvh.count: on the
    canonical tree's own export the counts and hits agree exactly."""
    sc, model, poses, _, _ = bench.raycast_workload("room_vlp16")
    poses = poses[:5]
    W, H = oracle.model_size(model)
    gids = np.arange(poses.shape[0] * W * H, dtype=np.uint64)[::3]
    o, d = oracle.Scene(sc.vertices, sc.faces).rays(model, IDENT, poses, gids)
    lb = oracle.CanonicalLbvh(sc.vertices, sc.faces)
    v1, t1, h1, f1 = lb.count(o, d, model.range.max)
    v2, t2, h2, f2 = oracle.tree_count(lb.export(), o, d, model.range.max)
    assert np.array_equal(v1, v2) and np.array_equal(t1, t2) and np.array_equal(f1, f2)
    assert np.array_equal(h1.view(np.uint32), h2.view(np.uint32))
