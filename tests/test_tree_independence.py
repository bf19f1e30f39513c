"""The closest hit does not depend on the tree: the same mesh under two topologies (the GPU LBVH
and the oracle's binned-SAH tree, one triangle per leaf, loaded as a map file) gives bit-identical
outputs for every walk.  This holds only if no box test culls a box that the ray truly meets:
scenes far from the coordinate origin (large |o/d| in the slab arithmetic) and grazing camera
rays are where a box test that is not conservative loses hits."""
import numpy as np
import pytest
import torch

import oracle
import rmagine_gb300 as rm
from rmagine_gb300 import scenes, sensors

pytestmark = pytest.mark.gpu

WALKS = {"per_ray": dict(packet=0), "packet": dict(packet=1), "wide": dict(bvh_width=4, packet=0),
         "wide8": dict(bvh_width=8, packet=0),
         "short_stack": dict(stack_depth=8, packet=0)}


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    torch.cuda.set_device(0)


def _translated(sc, dx, dy, dz=0.0):
    v = sc.vertices.astype(np.float64) + np.array([dx, dy, dz])
    return v.astype(np.float32), sc.faces


def _poses_translated(poses, dx, dy, dz=0.0):
    p = poses.copy()
    p[:, 4] += dx
    p[:, 5] += dy
    p[:, 6] += dz
    return p


def _both_maps(v, f, tmp_path):
    path = tmp_path / "sah.rmg"
    depth = oracle.Scene(v, f, max_leaf=1).save_map(path)
    return rm.Map(v, f).build_wide8(), rm.Map.load(path).build_wide8(), depth


def _run(m, model, poses, cfg):
    sim = rm.make_simulator(model, m)
    if cfg is not None:
        sim.launch_config = rm.launch_config(**cfg)
    res = sim.simulate(torch.from_numpy(np.ascontiguousarray(poses, np.float32)).cuda())
    torch.cuda.synchronize()
    return {a: getattr(res, a).cpu() for a in rm.ATTRIBUTES}


def _check(m1, m2, model, poses):
    for name, cfg in WALKS.items():
        a = _run(m1, model, poses, cfg)
        b = _run(m2, model, poses, cfg)
        for k in a:
            same = torch.equal(a[k].contiguous().view(torch.uint8), b[k].contiguous().view(torch.uint8))
            if not same:
                r1, r2 = a["ranges"].view(torch.int32), b["ranges"].view(torch.int32)
                n = int((r1 != r2).sum())
                raise AssertionError(f"{name}: {k} differs between the trees ({n} ranges differ)")
    assert m1.status() == 0 and m2.status() == 0


@pytest.mark.parametrize("offset", [0.0, 3000.0])
def test_terrain_far_from_origin_pinhole_and_spherical(tmp_path, offset):
    sc = scenes.terrain(grid=160, size=120.0, amplitude=8.0, n_boxes=80, seed=21)
    poses = scenes.terrain_poses(sc, 12, seed=22, size=120.0, above=0.8)
    v, f = _translated(sc, offset, -0.5 * offset, 0.25 * offset)
    poses = _poses_translated(poses, offset, -0.5 * offset, 0.25 * offset)
    lbvh, sah, depth = _both_maps(v, f, tmp_path)
    assert depth <= 64
    _check(lbvh, sah, sensors.depth_camera(160, 120, 100.0), poses)
    _check(lbvh, sah, sensors.ouster_like(rows=32, cols=512), poses)


def test_box_room_vlp16(tmp_path):
    sc = scenes.box_room(seed=23, n_boxes=120)
    v, f = _translated(sc, 500.0, 500.0)
    poses = _poses_translated(scenes.room_poses(16, seed=24), 500.0, 500.0)
    lbvh, sah, _ = _both_maps(v, f, tmp_path)
    _check(lbvh, sah, sensors.vlp16_900(), poses)
