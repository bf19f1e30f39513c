"""Instanced scenes (two-level BVH): the oracle's brute-force restatement pinned on the CPU, and
rmg_simulate_scene against it on the GPU.

rmagine builds such maps from files (make_embree_scene, EmbreeScene.cpp:326-406: one instance per
node with meshes, plain meshes added directly) and reports instance ids as ObjectIds and mesh ids
as GeomIds (SphereSimulatorEmbree.tcc:160-186); its own tests cover only single-mesh maps, so the
scene results are pinned here by (a) equality with the single-mesh path for identity instances,
(b) the reference's cube known answers through an instance, and (c) the brute-force oracle."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from oracle.scene import InstancedScene
from rmagine_gb300 import scenes, sensors, transforms

GOLD = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())
IDENT = transforms.identity()
ALL = ("hits", "ranges", "points", "normals", "face_ids", "geom_ids", "object_ids")


def quat(axis, angle):
    axis = np.asarray(axis, np.float64)
    axis = axis / np.linalg.norm(axis)
    return np.concatenate([axis * np.sin(angle / 2), [np.cos(angle / 2)]]).astype(np.float32)


def pose(q, t):
    T = IDENT.copy()
    T[:4] = q
    T[4:7] = t
    return T


def random_instances(n, n_geoms, seed, spread=8.0, scale_range=(0.5, 2.0)):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        q = rng.standard_normal(4)
        q = (q / np.linalg.norm(q)).astype(np.float32)
        t = rng.uniform(-spread, spread, 3).astype(np.float32)
        t[2] = rng.uniform(0.0, 3.0)
        s = rng.uniform(*scale_range, 3).astype(np.float32)
        out.append(dict(geometry=int(rng.integers(0, n_geoms)), T=pose(q, t), scale=s, geom_id=int(rng.integers(0, 4)),
                        object_id=100 + i))
    return out


def mesh_library():
    cube_v, cube_f = scenes.gen_cube()
    box_v, box_f = scenes.box_mesh([-0.3, -0.2, 0.0], [0.3, 0.2, 1.5])
    room = scenes.box_room(seed=4, n_boxes=6, half=3.0, height=2.5)
    return [(cube_v, cube_f), (box_v, box_f), (room.vertices, room.faces)]


# ---- CPU: pin the scene oracle -----------------------------------------------------------
def test_oracle_identity_instance_equals_the_single_mesh_path():
    room = scenes.box_room(seed=0, n_boxes=10)
    sc = InstancedScene([(room.vertices, room.faces)], [dict(geometry=0, T=IDENT, geom_id=0, object_id=0)])
    model = sensors.vlp16_900()
    poses = scenes.room_poses(2, seed=1)
    a = sc.simulate(model, IDENT, poses)
    b = oracle.Scene(room.vertices, room.faces).simulate(model, IDENT, poses)
    for k in ALL:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


@pytest.mark.parametrize("name", ["spherical_cube_range", "o1dn_cube_range", "ondn_cube_range"])
def test_oracle_cube_known_answers_through_an_instance(name):
    """The reference's genCube known answers, with the cube placed by an instance that rotates it
    by 90 deg about z and moves it by (5, -2, 1) and a sensor moved by the same transform."""
    g = GOLD[name]
    model = {"example_spherical": sensors.example_spherical, "example_o1dn": sensors.example_o1dn,
             "example_ondn": sensors.example_ondn}[g["model"]]()
    v, f = scenes.gen_cube()
    Tinst = pose(quat([0, 0, 1], np.pi / 2), [5.0, -2.0, 1.0])
    sc = InstancedScene([(v, f)], [dict(geometry=0, T=Tinst, object_id=7)])
    res = sc.simulate(model, IDENT, Tinst[None])
    W, H = oracle.model_size(model)
    if g.get("vid") == "phi.size/2":
        gid = (H // 2) * W + int(g["hid"])
    else:
        gid = int(g.get("ray", 0))
    assert abs(float(res["ranges"][gid]) - g["expect"]) < g["tol"]
    assert res["object_ids"][gid] == 7


def test_oracle_nearest_instance_wins_and_ids_follow_it():
    v, f = scenes.gen_cube()
    insts = [dict(geometry=0, T=pose(IDENT[:4], [4.0, 0, 0]), geom_id=1, object_id=11),
             dict(geometry=0, T=pose(IDENT[:4], [2.0, 0, 0]), scale=(0.5, 0.5, 0.5), geom_id=2, object_id=22)]
    sc = InstancedScene([(v, f)], insts)
    model = sensors.OnDnModel(width=1, height=1, range=sensors.Interval(0.0, 100.0),
                              origs=np.zeros((1, 3), np.float32), dirs=np.array([[1, 0, 0]], np.float32))
    r = sc.simulate(model, IDENT, IDENT[None])
    # the half-size cube at x = 2 has its near face at x = 1.75
    assert abs(float(r["ranges"][0]) - 1.75) < 1e-6
    assert r["object_ids"][0] == 22 and r["geom_ids"][0] == 2
    assert np.allclose(r["normals"][0], [-1, 0, 0])


def test_oracle_scaled_rotated_instance_matches_a_baked_mesh():
    """An instance equals the same mesh with its vertices moved by T * diag(s) up to binary32
    rounding (the ray is transformed instead of the mesh)."""
    v, f = scenes.gen_cube()
    T = pose(quat([1, 2, 3], 0.7), [1.0, -3.0, 0.5])
    s = np.array([2.0, 0.5, 1.5], np.float32)
    sc = InstancedScene([(v, f)], [dict(geometry=0, T=T, scale=s)])
    baked = transforms.apply(T[None], (v * s).astype(np.float32))
    plain = oracle.Scene(baked, f)
    model = sensors.vlp16_900()
    P = np.stack([pose(IDENT[:4], [1.0 - 5.0, -3.0, 0.5]), pose(IDENT[:4], [1.0 + 5.0, -3.0, 0.5]),
                  pose(quat([0, 0, 1], 1.0), [1.0, 2.0, 0.5])])
    a = sc.simulate(model, IDENT, P)
    b = plain.simulate(model, IDENT, P)
    same = a["face_ids"] == b["face_ids"]
    assert same.mean() > 0.999 and a["hits"].sum() > 1000
    assert np.abs(a["ranges"][same] - b["ranges"][same]).max() < 1e-4
    hit = same & (a["hits"] > 0)
    assert np.abs(a["normals"][hit] - b["normals"][hit]).max() < 1e-5


# ---- GPU ---------------------------------------------------------------------------------
def _gpu_scene(meshes, insts):
    import rmagine_gb300 as rm

    geoms = [rm.Map(v, f) for v, f in meshes]
    return rm.Scene(geoms, [rm.Instance(i["geometry"], i["T"], i.get("scale", (1, 1, 1)), i.get("geom_id", 0),
                                        i.get("object_id", 0)) for i in insts])


def _run(scene, model, poses, attrs=ALL, Tsb=IDENT):
    import torch

    import rmagine_gb300 as rm

    sim = rm.make_simulator(model, scene)
    sim.setTsb(Tsb)
    res = sim.simulate(torch.from_numpy(np.ascontiguousarray(poses, np.float32)).cuda(), attrs=attrs)
    torch.cuda.synchronize()
    out = {}
    for a in attrs:
        t = getattr(res, a).cpu().numpy()
        out[a] = t.view(np.uint32) if a in ("face_ids", "geom_ids", "object_ids") else t
    return out


def _agree(got, want, rep):
    """Exact equality of every attribute on the rays the certifier did not dispute."""
    bad = (got["face_ids"] != want["face_ids"]) | (got["object_ids"] != want["object_ids"]) | \
        (np.abs(got["ranges"].astype(np.float64) - want["ranges"].astype(np.float64)) > 1e-4)
    ok = ~bad
    assert rep["unexcused"] == 0, rep
    for k in got:
        assert np.array_equal(got[k][ok], want[k][ok], equal_nan=True), k


@pytest.mark.gpu
def test_identity_instance_scene_equals_the_map_bitwise(built):
    import torch

    import rmagine_gb300 as rm

    torch.cuda.set_device(0)
    room = scenes.box_room(seed=0, n_boxes=30)
    model = sensors.vlp16_900()
    poses = scenes.room_poses(8, seed=1)
    scene = _gpu_scene([(room.vertices, room.faces)], [dict(geometry=0, T=IDENT, geom_id=3, object_id=9)])
    a = _run(scene, model, poses)
    b = _run(rm.Map(room.vertices, room.faces), model, poses)
    hit = b["face_ids"] != 0xFFFFFFFF
    for k in ("hits", "ranges", "points", "normals", "face_ids"):
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    assert np.all(a["geom_ids"][hit] == 3) and np.all(a["object_ids"][hit] == 9)
    assert np.all(a["geom_ids"][~hit] == 0xFFFFFFFF)
    assert scene.status() == 0


def _models():
    rng = np.random.default_rng(3)
    d = rng.standard_normal((4096, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return {"spherical": sensors.vlp16_900(), "pinhole": sensors.depth_camera(200, 150),
            "o1dn": sensors.O1DnModel(width=4096, height=1, range=sensors.Interval(0.2, 80.0), orig=(0.05, 0.0, 0.1),
                                      dirs=d),
            "ondn": sensors.OnDnModel(width=2048, height=2, range=sensors.Interval(0.2, 80.0),
                                      origs=rng.uniform(-0.1, 0.1, (4096, 3)).astype(np.float32), dirs=d)}


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["spherical", "pinhole", "o1dn", "ondn"])
def test_random_instanced_scene_matches_the_oracle(built, kind):
    import torch

    torch.cuda.set_device(0)
    meshes = mesh_library()
    insts = random_instances(40, len(meshes), seed=5)
    scene = _gpu_scene(meshes, insts)
    model = _models()[kind]
    poses = np.stack([pose(quat([0, 0, 1], a), [np.cos(a) * 3, np.sin(a) * 3, 1.2])
                      for a in np.linspace(0, 2 * np.pi, 4, endpoint=False)])
    got = _run(scene, model, poses)
    osc = InstancedScene(meshes, insts)
    want = osc.simulate(model, IDENT, poses)
    assert got["hits"].sum() > 0.05 * got["hits"].size
    assert len(np.unique(got["object_ids"])) >= 6
    rep = osc.certify(model, IDENT, poses, got, want)
    _agree(got, {k: want[k] for k in got}, rep)
    assert scene.status() == 0


@pytest.mark.gpu
def test_update_refit_and_rebuild_follow_moving_instances(built):
    import torch

    import rmagine_gb300 as rm

    torch.cuda.set_device(0)
    meshes = mesh_library()
    insts = random_instances(24, len(meshes), seed=8)
    scene = _gpu_scene(meshes, insts)
    model = sensors.vlp16_900()
    poses = np.stack([pose(IDENT[:4], [0.0, 0.0, 1.0]), pose(quat([0, 0, 1], 1.0), [2.0, 1.0, 1.5])])
    moved = random_instances(24, len(meshes), seed=9)
    for i, m in enumerate(moved):
        m["geometry"] = insts[i]["geometry"]
    new = [rm.Instance(m["geometry"], m["T"], m["scale"], m["geom_id"], m["object_id"]) for m in moved]
    scene.update(new)                      # refit
    a = _run(scene, model, poses)
    scene.update(new, rebuild=True)        # rebuild
    b = _run(scene, model, poses)
    for k in ALL:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    osc = InstancedScene(meshes, moved)
    want = osc.simulate(model, IDENT, poses)
    _agree(a, {k: want[k] for k in a}, osc.certify(model, IDENT, poses, a, want))


@pytest.mark.gpu
def test_geometry_refit_then_scene_update(built):
    import torch

    import rmagine_gb300 as rm

    torch.cuda.set_device(0)
    v, f = scenes.gen_cube()
    g = rm.Map(v, f)
    insts = [rm.Instance(0, pose(IDENT[:4], [3.0, 0, 0]), object_id=1),
             rm.Instance(0, pose(IDENT[:4], [-3.0, 0, 0]), object_id=2)]
    scene = rm.Scene([g], insts)
    model = sensors.vlp16_900()
    v2 = (v * np.float32(2.0)).astype(np.float32)  # the mesh grows: bounds change
    g.refit(v2)
    scene.update(insts)
    got = _run(scene, model, IDENT[None])
    osc = InstancedScene([(v2, f)], [dict(geometry=0, T=i.T, object_id=i.object_id) for i in insts])
    want = osc.simulate(model, IDENT, IDENT[None])
    _agree(got, {k: want[k] for k in got}, osc.certify(model, IDENT, IDENT[None], got, want))


@pytest.mark.gpu
def test_empty_scenes_and_bad_instances(built):
    import torch

    import rmagine_gb300 as rm

    torch.cuda.set_device(0)
    model = sensors.vlp16_900()
    empty = rm.Scene([], [])
    r = _run(empty, model, IDENT[None])
    assert r["hits"].sum() == 0 and np.all(r["face_ids"] == 0xFFFFFFFF)
    assert np.all(r["ranges"] == np.float32(model.range.max) + np.float32(1))
    g0 = rm.Map(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
    only_empty = rm.Scene([g0], [rm.Instance(0)])
    assert _run(only_empty, model, IDENT[None])["hits"].sum() == 0
    v, f = scenes.gen_cube()
    g = rm.Map(v, f)
    for bad in (rm.Instance(1), rm.Instance(0, scale=(1.0, 0.0, 1.0)),
                rm.Instance(0, T=np.array([0, 0, 0, 2, 0, 0, 0, 0], np.float32))):
        with pytest.raises(rm.RmgError):
            rm.Scene([g], [bad])
    sc = rm.Scene([g], [rm.Instance(0)])
    with pytest.raises(rm.RmgError):
        sc.update([rm.Instance(0), rm.Instance(0)])


def test_oracle_instanced_terrain_equals_the_baked_terrain():
    """scenes.instanced_terrain places the boxes by instances; ranges agree with the baked mesh
    to binary32 rounding, and box hits report object ids 1 + box index."""
    meshes, insts, baked = scenes.instanced_terrain(grid=64, n_boxes=60, seed=3, size=60.0)
    osc = InstancedScene(meshes, insts)
    model = sensors.vlp16_900()
    P = scenes.terrain_poses(baked, 3, seed=4, size=60.0)
    a = osc.simulate(model, IDENT, P)
    b = oracle.Scene(baked.vertices, baked.faces).simulate(model, IDENT, P)
    both = (a["hits"] > 0) & (b["hits"] > 0)
    assert both.mean() > 0.4
    close = np.abs(a["ranges"][both] - b["ranges"][both]) < 1e-4
    assert close.mean() > 0.999
    n_terrain = meshes[0][1].shape[0]
    on_box = both & (b["face_ids"] >= n_terrain)
    box_of_face = (b["face_ids"][on_box] - n_terrain) // 12
    agree = a["object_ids"][on_box] == 1 + box_of_face
    assert on_box.sum() > 20 and agree.mean() > 0.99


# ---- opened trees (partial re-braiding) ----------------------------------------------------
# A geometry of at least 2 x 16,384 triangles enters the top tree as pieces of its own tree; the
# results must be those of the unopened tree: bit-equal to the single-mesh path for an identity
# instance, and the oracle's (which tries every instance whole) under rotated, scaled instances.
def _opened_terrain(grid=256, size=120.0, n_boxes=0, seed=21):
    sc = scenes.terrain(grid=grid, size=size, n_boxes=n_boxes, seed=seed)
    assert sc.faces.shape[0] >= 4 * 16384  # opened into several pieces
    return sc


@pytest.mark.gpu
def test_opened_tree_identity_instance_equals_the_map_bitwise(built):
    import torch

    import rmagine_gb300 as rm

    torch.cuda.set_device(0)
    sc = _opened_terrain()
    model = sensors.ouster_like(rows=32, cols=512)
    poses = scenes.terrain_poses(sc, 6, seed=22, size=120.0)
    scene = _gpu_scene([(sc.vertices, sc.faces)], [dict(geometry=0, T=IDENT, geom_id=2, object_id=5)])
    a = _run(scene, model, poses)
    b = _run(rm.Map(sc.vertices, sc.faces), model, poses)
    hit = b["face_ids"] != 0xFFFFFFFF
    assert hit.mean() > 0.5
    for k in ("hits", "ranges", "points", "normals", "face_ids"):
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    assert np.all(a["object_ids"][hit] == 5) and np.all(a["object_ids"][~hit] == 0xFFFFFFFF)
    assert scene.status() == 0


def _opened_scene_instances(sc):
    cube_v, cube_f = scenes.gen_cube()
    insts = [dict(geometry=0, T=pose(quat([0, 0, 1], 0.5), [3.0, -2.0, 0.5]), scale=np.array([1.0, 1.2, 0.8], np.float32),
                  geom_id=0, object_id=1),
             dict(geometry=0, T=pose(quat([0.2, 1, 0], 3.0), [0.0, 0.0, 14.0]), scale=np.array([0.5, 0.5, 0.5], np.float32),
                  geom_id=0, object_id=2)]
    rng = np.random.default_rng(23)
    for i in range(40):
        t = np.array([*rng.uniform(-40, 40, 2), rng.uniform(0.0, 6.0)], np.float32)
        insts.append(dict(geometry=1, T=pose(quat(rng.standard_normal(3), rng.uniform(0, 6)), t),
                          scale=rng.uniform(0.5, 3.0, 3).astype(np.float32), geom_id=1, object_id=10 + i))
    return [(sc.vertices, sc.faces), (cube_v, cube_f)], insts


@pytest.mark.gpu
def test_opened_tree_under_rotated_scaled_instances_matches_the_oracle(built):
    import torch

    torch.cuda.set_device(0)
    sc = _opened_terrain()
    meshes, insts = _opened_scene_instances(sc)
    scene = _gpu_scene(meshes, insts)
    model = sensors.ouster_like(rows=32, cols=512)
    poses = np.stack([pose(quat([0, 0, 1], a), [np.cos(a) * 20, np.sin(a) * 20, 8.0])
                      for a in np.linspace(0, 2 * np.pi, 5, endpoint=False)])
    got = _run(scene, model, poses)
    osc = InstancedScene(meshes, insts)
    want = osc.simulate(model, IDENT, poses)
    assert got["hits"].mean() > 0.3
    assert len(np.unique(got["object_ids"])) >= 10
    rep = osc.certify(model, IDENT, poses, got, want)
    _agree(got, {k: want[k] for k in got}, rep)
    assert scene.status() == 0


@pytest.mark.gpu
def test_opened_tree_follows_a_geometry_refit(built):
    """The pieces keep their nodes after a refit of the geometry; the scene update takes their new
    boxes from the refitted tree."""
    import torch

    import rmagine_gb300 as rm

    torch.cuda.set_device(0)
    sc = _opened_terrain()
    meshes, insts = _opened_scene_instances(sc)
    geoms = [rm.Map(v, f) for v, f in meshes]
    objs = [rm.Instance(i["geometry"], i["T"], i["scale"], i["geom_id"], i["object_id"]) for i in insts]
    scene = rm.Scene(geoms, objs)
    v2 = sc.vertices.copy()
    v2[:, 2] = v2[:, 2] * np.float32(1.7) + np.float32(1.0)  # heights change: every piece's box moves
    geoms[0].refit(v2)
    scene.update(objs)
    model = sensors.ouster_like(rows=32, cols=512)
    poses = np.stack([pose(quat([0, 0, 1], a), [np.cos(a) * 15, np.sin(a) * 15, 20.0])
                      for a in np.linspace(0, 2 * np.pi, 4, endpoint=False)])
    got = _run(scene, model, poses)
    meshes2 = [(v2, sc.faces), meshes[1]]
    osc = InstancedScene(meshes2, insts)
    want = osc.simulate(model, IDENT, poses)
    assert got["hits"].mean() > 0.3
    _agree(got, {k: want[k] for k in got}, osc.certify(model, IDENT, poses, got, want))
    assert scene.status() == 0


# ---- identity instances walked directly (outside the top tree) -----------------------------
def _mixed_identity_instances():
    """Identity instances of three geometries (one of them twice, the duplicate with a larger index
    and other ids), between rotated and scaled instances."""
    rest = random_instances(12, 3, seed=31)
    ident = lambda g, oid: dict(geometry=g, T=IDENT.copy(), scale=np.ones(3, np.float32), geom_id=g, object_id=oid)
    return rest[:4] + [ident(2, 1)] + rest[4:8] + [ident(0, 2), ident(2, 3), ident(1, 4)] + rest[8:]


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["spherical", "o1dn"])
def test_identity_instances_walked_directly_match_the_oracle(built, kind):
    import torch

    torch.cuda.set_device(0)
    meshes = mesh_library()
    insts = _mixed_identity_instances()
    scene = _gpu_scene(meshes, insts)
    model = _models()[kind]
    poses = np.stack([pose(quat([0, 0, 1], a), [np.cos(a) * 1.5, np.sin(a) * 1.5, 1.0])
                      for a in np.linspace(0, 2 * np.pi, 4, endpoint=False)])
    got = _run(scene, model, poses)
    osc = InstancedScene(meshes, insts)
    want = osc.simulate(model, IDENT, poses)
    assert np.any(got["object_ids"] == 1) and not np.any(got["object_ids"] == 3)  # the duplicate never wins
    rep = osc.certify(model, IDENT, poses, got, want)
    _agree(got, {k: want[k] for k in got}, rep)
    assert scene.status() == 0


@pytest.mark.gpu
def test_instances_leaving_and_entering_the_identity_follow_the_oracle(built):
    import torch

    import rmagine_gb300 as rm

    torch.cuda.set_device(0)
    meshes = mesh_library()
    insts = _mixed_identity_instances()
    scene = _gpu_scene(meshes, insts)
    model = sensors.vlp16_900()
    poses = np.stack([pose(IDENT[:4], [0.3, 0.2, 1.0]), pose(quat([0, 0, 1], 2.0), [-1.0, 0.5, 1.2])])
    steps = []
    moved = [dict(i) for i in insts]
    moved[4] = dict(moved[4], T=pose(quat([0, 0, 1], 0.3), [0.5, 0.0, 0.0]))  # the room leaves the identity
    steps.append(moved)
    back = [dict(i) for i in moved]
    back[4] = dict(back[4], T=IDENT.copy())                                     # and comes back
    back[9] = dict(back[9], T=pose(quat([1, 0, 0], 0.2), [0.0, 0.0, 0.2]))     # the cube leaves it
    steps.append(back)
    for step in steps:
        for rebuild in (False, True):
            scene.update([rm.Instance(i["geometry"], i["T"], i.get("scale", (1, 1, 1)), i.get("geom_id", 0),
                                      i.get("object_id", 0)) for i in step], rebuild=rebuild)
            got = _run(scene, model, poses)
            osc = InstancedScene(meshes, step)
            want = osc.simulate(model, IDENT, poses)
            _agree(got, {k: want[k] for k in got}, osc.certify(model, IDENT, poses, got, want))
    assert scene.status() == 0


@pytest.mark.gpu
def test_more_identity_geometries_than_walked_directly(built):
    import torch

    torch.cuda.set_device(0)
    meshes = []
    for k in range(6):  # six small rooms side by side: the first four walked directly, the rest in the tree
        room = scenes.box_room(seed=40 + k, n_boxes=3, half=1.5, height=2.0)
        meshes.append(((room.vertices + np.array([4.0 * k, 0, 0], np.float32)).astype(np.float32), room.faces))
    insts = [dict(geometry=k, T=IDENT.copy(), scale=np.ones(3, np.float32), geom_id=k, object_id=k)
             for k in range(6)]
    scene = _gpu_scene(meshes, insts)
    model = sensors.vlp16_900()
    poses = np.stack([pose(IDENT[:4], [4.0 * k, 0.2, 1.0]) for k in range(6)])
    got = _run(scene, model, poses)
    osc = InstancedScene(meshes, insts)
    want = osc.simulate(model, IDENT, poses)
    assert len(np.unique(got["object_ids"][got["hits"] > 0])) == 6
    _agree(got, {k: want[k] for k in got}, osc.certify(model, IDENT, poses, got, want))
