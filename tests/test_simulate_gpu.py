"""GPU parity of the plain simulate path against the oracle (through the C ABI).

Bar: hits, face ids and ranges bit-identical to the oracle on every ray except
rays the binary64 certifier excuses (edge band 1e-6 barycentric, t ties,
range bounds); points and normals bit-identical wherever the face agrees.
"""
import json
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle
import rmagine_gb300 as rm
from rmagine_gb300 import _lib, scenes, sensors

pytestmark = pytest.mark.gpu

GOLD = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())
IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)
ALL = rm.ATTRIBUTES


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    torch.cuda.set_device(0)


def gpu_sim(map_, model, Tbm, Tsb=IDENT, attrs=ALL, cfg=None):
    sim = rm.make_simulator(model, map_)
    sim.setTsb(Tsb)
    if cfg is not None:
        sim.launch_config = cfg
    res = sim.simulate(torch.from_numpy(np.ascontiguousarray(Tbm, np.float32)).cuda(), attrs=attrs)
    torch.cuda.synchronize()
    out = {}
    for a in attrs:
        t = getattr(res, a).cpu().numpy()
        out[a] = t.view(np.uint32) if a.endswith("_ids") else t
    return out


def same_float(a, b):
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


def check_parity(scene_v, scene_f, model, Tbm, Tsb=IDENT, attrs=ALL, max_disputed_frac=1e-3):
    m = rm.Map(scene_v, scene_f)
    got = gpu_sim(m, model, Tbm, Tsb, attrs)
    assert m.status() == 0
    sc = oracle.Scene(scene_v, scene_f)
    want = sc.simulate(model, Tsb, Tbm, attrs=attrs)
    rep = oracle.certify(sc, model, Tsb, Tbm, got, want)
    assert rep["unexcused"] == 0, rep
    assert rep["disputed"] <= max_disputed_frac * rep["rays"], rep
    agree = got["face_ids"] == want["face_ids"]
    for a in ("hits", "ranges", "geom_ids", "object_ids"):
        if a in attrs:
            assert np.array_equal(got[a][agree].view(np.uint8 if a == "hits" else np.uint32),
                                  want[a][agree].view(np.uint8 if a == "hits" else np.uint32)), a
    for a in ("points", "normals"):
        if a in attrs:
            assert same_float(got[a][agree], want[a][agree]), a
    return got, want, rep


# ---- known answers of the reference's tests, on the GPU ------------------------------
def cube_map():
    v, f = scenes.gen_cube()
    return rm.Map(v, f)


def test_known_answer_spherical():
    g = GOLD["spherical_cube_range"]
    m = sensors.example_spherical()
    r = gpu_sim(cube_map(), m, np.tile(IDENT, (100, 1)))["ranges"]
    assert abs(r[99 * m.size() + m.getBufferId(m.phi.size // 2, 0)] - g["expect"]) <= g["tol"]


def test_known_answer_pinhole():
    g = GOLD["pinhole_cube_point"]
    m = sensors.example_pinhole()
    res = gpu_sim(cube_map(), m, np.tile(IDENT, (100, 1)))
    p = oracle.directions(m)[0] * res["ranges"][99 * m.size()]
    assert np.abs(p - np.array(g["expect"])).sum() <= g["tol"]
    assert np.abs(res["points"][99 * m.size()] - np.array(g["expect"])).sum() <= g["tol"]


def test_known_answer_o1dn():
    m = sensors.example_o1dn()
    res = gpu_sim(cube_map(), m, np.tile(IDENT, (100, 1)))
    k = 99 * m.size()
    assert np.abs(res["points"][k] - np.array(GOLD["o1dn_cube_point"]["expect"])).sum() <= 1e-4
    assert np.linalg.norm(res["normals"][k] - np.array(GOLD["o1dn_cube_normal"]["expect"])) <= 1e-4
    assert abs(res["ranges"][k] - GOLD["o1dn_cube_range"]["expect"]) <= 1e-4


def test_known_answer_ondn():
    m1 = sensors.OnDnModel(width=1, height=1, range=sensors.Interval(0.0, 100.0),
                           origs=np.zeros((1, 3), np.float32), dirs=np.array([[1, 0, 0]], np.float32))
    assert abs(gpu_sim(cube_map(), m1, np.tile(IDENT, (100, 1)))["ranges"][0] - 0.5) <= 1e-4
    m = sensors.example_ondn()
    r = gpu_sim(cube_map(), m, np.tile(IDENT, (100, 1)))["ranges"]
    assert abs(r[99 * m.size()] - GOLD["ondn_cube_range"]["expect"]) <= 1e-4


# ---- building blocks ----------------------------------------------------------------
@pytest.mark.parametrize("model", ["vlp16_900", "ouster_like", "example_pinhole", "depth_camera"])
def test_direction_table_matches_oracle(model):
    m = getattr(sensors, model)()
    s = rm.Sensor(m)
    assert np.array_equal(s.directions(), oracle.directions(m))


@pytest.mark.parametrize("which", ["room", "terrain", "duplicates"])
def test_lbvh_matches_canonical_build(which):
    if which == "room":
        sc = scenes.box_room(seed=0, n_boxes=200)
        v, f = sc.vertices, sc.faces
    elif which == "terrain":
        sc = scenes.terrain(grid=96, n_boxes=100, seed=3)
        v, f = sc.vertices, sc.faces
    else:  # many identical triangles: equal Morton codes, index tie-break
        v, f = scenes.gen_cube()
        v, f = scenes.merge([(v, f)] * 40)
    m = rm.Map(v, f, builder="lbvh")
    g = m.export()
    c = oracle.CanonicalLbvh(v, f).export()
    assert np.array_equal(g["leaf_order"], c["leaf_order"])
    assert np.array_equal(g["links"], c["links"])
    assert same_float(g["boxes"], c["boxes"])
    assert same_float(g["tris"], c["tris"])
    info = m.info()
    assert info["n_faces"] == f.shape[0] and info["n_nodes"] == f.shape[0] - 1
    assert info["depth"] >= int(np.ceil(np.log2(f.shape[0])))


# ---- parity on the workloads' scenes -------------------------------------------------------
def test_parity_room_vlp16_all_attributes():
    sc = scenes.box_room(seed=0, n_boxes=200)
    assert sc.n_faces == 2412
    check_parity(sc.vertices, sc.faces, sensors.vlp16_900(), scenes.room_poses(100, seed=1))


def test_parity_terrain_ouster_and_pinhole():
    sc = scenes.terrain(grid=128, n_boxes=200, seed=5)
    poses = scenes.terrain_poses(sc, 6, seed=6)
    check_parity(sc.vertices, sc.faces, sensors.ouster_like(), poses)
    check_parity(sc.vertices, sc.faces, sensors.depth_camera(160, 120), poses)


def test_parity_o1dn_ondn_with_sensor_offset():
    sc = scenes.terrain(grid=96, n_boxes=100, seed=7)
    poses = scenes.terrain_poses(sc, 5, seed=8)
    Tsb = np.array([0, 0, np.sin(0.05), np.cos(0.05), 0.1, 0.0, 0.2, 0], np.float32)
    o1 = sensors.O1DnModel(width=1000, height=1, range=sensors.Interval(0.2, 130.0), orig=(0.1, 0.0, 0.2),
                           dirs=sensors.sphere_directions(1000, seed=9))
    check_parity(sc.vertices, sc.faces, o1, poses, Tsb)
    rng = np.random.default_rng(10)
    on = sensors.OnDnModel(width=50, height=20, range=sensors.Interval(0.0, 130.0),
                           origs=rng.uniform(-0.5, 0.5, (1000, 3)).astype(np.float32),
                           dirs=sensors.sphere_directions(1000, seed=11))
    check_parity(sc.vertices, sc.faces, on, poses, Tsb)


# ---- launch variants are bit-identical ----------------------------------------------------
def test_stack_depths_and_tiles_bitwise_identical():
    sc = scenes.terrain(grid=128, n_boxes=200, seed=12)
    poses = scenes.terrain_poses(sc, 4, seed=13)
    m = rm.Map(sc.vertices, sc.faces).build_wide8()
    model = sensors.ouster_like(64, 512)
    base = gpu_sim(m, model, poses, cfg=rm.launch_config(8, 4, 8, 4, bvh_width=2))
    assert m.info()["depth"] <= 32
    for cfg in [(0, 4, 8, 4, 0, 4, 2), (16, 2, 8, 4, 0, 4, 2), (16, 8, 32, 1, 0, 4, 2), (8, 1, 4, 8, 0, 4, 2),
                (8, 4, 16, 2, 0, 4, 2), (0, 8, 2, 16, 0, 4, 2),
                (16, 4, 8, 4, 0, 4, 4), (16, 2, 16, 2, 0, 4, 4), (16, 8, 32, 1, 0, 4, 4), (16, 4, 8, 4),
                (16, 4, 8, 4, 0, 4, 2, 1), (16, 2, 16, 2, 0, 4, 2, 1), (16, 8, 32, 1, 0, 4, 2, 1),
                (16, 4, 4, 8, 0, 4, 0, 1),
                (16, 4, 8, 4, 0, 4, 8), (16, 2, 16, 2, 0, 4, 8), (16, 8, 4, 8, 0, 4, 8),
                (8, 4, 8, 4, 16, 4), (16, 2, 8, 4, 32, 1), (8, 8, 16, 2, 1, 7), (16, 4, 4, 8, 24, 64)]:
        other = gpu_sim(m, model, poses, cfg=rm.launch_config(*cfg))
        for a in ALL:
            assert np.array_equal(base[a].view(np.uint8), other[a].view(np.uint8)), (cfg, a)


def comb_mesh(extra_at_deepest=0):
    """Tiny triangles whose centroids sit at 2^i on each axis (i = 0..19): their Morton codes are
    single bits, so the radix tree is a chain (depth ~55, beyond the 32-level full stack); with
    `extra_at_deepest` more triangles on the first centroid the duplicate keys add index-split
    levels below it (depth > 64: the 128-bit trail)."""
    pts = [np.eye(3)[a] * 2.0 ** i for i in range(20) for a in range(3)] + [np.full(3, 2.0 ** 20)]
    pts += [pts[0]] * extra_at_deepest
    s = 0.05
    v = np.concatenate([[p + [-s, -s, 0], p + [s, -s, 0], p + [0, s, 0]] for p in pts]).astype(np.float32)
    f = np.arange(3 * len(pts), dtype=np.uint32).reshape(-1, 3)
    return v, f, np.array(pts[:61], np.float32)


@pytest.mark.parametrize("extra,min_depth,max_depth", [(0, 33, 64), (2048, 65, 128)])
def test_deep_trees_trail_walks(extra, min_depth, max_depth):
    """Trees deeper than the 32-level full stack run the trail walks (64- and 128-bit trails with
    the short stack or none): parity with the oracle, and every stack setting bit-identical."""
    v, f, centres = comb_mesh(extra)
    m = rm.Map(v, f, builder="lbvh")
    depth = m.info()["depth"]
    assert min_depth <= depth <= max_depth, depth
    origin = np.array([-3.0, -2.0, -1.0], np.float32)
    dirs = centres - origin
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rng = np.random.default_rng(4)
    rnd = rng.standard_normal((195, 3)).astype(np.float32)
    rnd /= np.linalg.norm(rnd, axis=1, keepdims=True)
    d = np.concatenate([dirs, rnd]).astype(np.float32)
    model = sensors.OnDnModel(width=64, height=4, range=sensors.Interval(0.0, 4.0e6),
                              origs=np.tile(origin, (256, 1)), dirs=d)
    poses = np.tile(IDENT, (3, 1))
    poses[1, 4:7] = (0.5, -0.25, 0.125)
    poses[2, :4] = scenes.euler_to_quat([0.0], [0.0], [0.01])[0]
    got, _, _ = check_parity(v, f, model, poses)
    assert got["hits"][:61].sum() >= 55  # the aimed rays reach their triangles
    for cfg in [(0, 4, 8, 4), (8, 4, 8, 4), (16, 2, 16, 2), (16, 4, 8, 4, 16, 2), (16, 4, 8, 4, 0, 4, 4)]:
        other = gpu_sim(m, model, poses, cfg=rm.launch_config(*cfg))
        for a in ALL:
            assert np.array_equal(got[a].view(np.uint8), other[a].view(np.uint8)), (cfg, a)
    assert m.status() == 0


# ---- edge cases -----------------------------------------------------------------------------
def test_empty_map_writes_misses():
    m = rm.Map(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
    model = sensors.vlp16_900()
    res = gpu_sim(m, model, scenes.room_poses(2))
    assert np.all(res["hits"] == 0)
    assert np.all(res["ranges"] == np.float32(131.0))
    assert np.all(np.isnan(res["points"])) and np.all(np.isnan(res["normals"]))
    assert np.all(res["face_ids"] == 0xFFFFFFFF)


def test_single_triangle_map():
    v = np.array([[2, -1, -1], [2, 1, -1], [2, 0, 1]], np.float32)
    f = np.array([[0, 1, 2]], np.uint32)
    check_parity(v, f, sensors.vlp16_900(), np.tile(IDENT, (2, 1)))


def test_ragged_tiles_and_single_pose():
    """Sensor sizes that are not multiples of the tile (W=37, H=5) and one pose, in both the
    one-tile-per-warp and the lane-refill launch modes."""
    sc = scenes.box_room(seed=2, n_boxes=30)
    m = sensors.SphericalModel(phi=sensors.DiscreteInterval(-0.2, 0.1, 5),
                               theta=sensors.DiscreteInterval(-3.0, 0.16, 37), range=sensors.Interval(0.1, 50.0))
    got, _, _ = check_parity(sc.vertices, sc.faces, m, scenes.room_poses(1, seed=3))
    mp = rm.Map(sc.vertices, sc.faces)
    for cfg in [(8, 4, 8, 4, 32, 1), (16, 2, 8, 4, 8, 3), (16, 4, 8, 4, 0, 4, 2, 1), (16, 4, 16, 2, 0, 4, 4, 0)]:
        other = gpu_sim(mp, m, scenes.room_poses(1, seed=3), cfg=rm.launch_config(*cfg))
        for a in ALL:
            assert np.array_equal(got[a].view(np.uint8), other[a].view(np.uint8)), (cfg, a)


def test_refill_mode_on_empty_map_and_corrupt_tree():
    model = sensors.vlp16_900()
    empty = rm.Map(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
    res = gpu_sim(empty, model, scenes.room_poses(2), cfg=rm.launch_config(8, 4, 8, 4, 16, 2))
    assert np.all(res["hits"] == 0) and np.all(res["face_ids"] == 0xFFFFFFFF)
    sc = scenes.box_room(seed=8, n_boxes=20)
    m = rm.Map(sc.vertices, sc.faces)
    g = m.export()
    internal = int(g["links"][0][0]) if g["links"][0][0] >= 0 else int(g["links"][0][1])
    _lib.call("rmg_map_debug_set_child", m.handle, internal, 0, 0)
    gpu_sim(m, model, scenes.room_poses(2, seed=9), attrs=("ranges",), cfg=rm.launch_config(16, 4, 8, 4, 32, 4))
    assert m.status(clear=True) == _lib.RMG_ERR_TRAVERSAL_BUDGET


def test_zero_poses_and_no_outputs_are_noops():
    sc = scenes.box_room(seed=2, n_boxes=5)
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.SphereSimulator(m)
    sim.setModel(sensors.vlp16_900())
    b = rm.Bundle("ranges")
    rm.resize_memory_bundle(b, 900, 16, 0)
    sim.simulate(torch.zeros((0, 8), device="cuda"), b)
    empty = rm.Bundle()
    sim.simulate(torch.from_numpy(scenes.room_poses(1)).cuda(), empty)
    torch.cuda.synchronize()


def test_host_bundle_matches_device_bundle():
    sc = scenes.box_room(seed=4, n_boxes=50)
    m = rm.Map(sc.vertices, sc.faces)
    model = sensors.vlp16_900()
    poses = scenes.room_poses(3, seed=5)
    dev = gpu_sim(m, model, poses)
    sim = rm.SphereSimulator(m)
    sim.setModel(model)
    hb = rm.resize_memory_bundle(rm.IntAttrAll(), 900, 16, 3, device="cpu", pin_memory=True)
    sim.simulate(torch.from_numpy(poses), hb)
    for a in ALL:
        assert np.array_equal(getattr(hb, a).numpy().view(np.uint8), dev[a].view(np.uint8)), a


@pytest.mark.parametrize("builder", ["lbvh", "sah"])
def test_refit_moves_geometry(builder):
    sc = scenes.box_room(seed=6, n_boxes=60)
    m = rm.Map(sc.vertices, sc.faces, builder=builder).build_wide8()
    links = m.export()["links"]
    moved = sc.vertices + np.array([0.3, -0.2, 0.1], np.float32)
    m.refit(moved)
    model = sensors.vlp16_900()
    poses = scenes.room_poses(4, seed=7)
    got = gpu_sim(m, model, poses)
    # the 8-wide tree (boxes and triangle copy) follows the refit
    wide8 = gpu_sim(m, model, poses, cfg=rm.launch_config(bvh_width=8, packet=0))
    for a in ALL:
        assert np.array_equal(wide8[a].view(np.uint8), got[a].view(np.uint8)), a
    sc2 = oracle.Scene(moved, sc.faces)
    want = sc2.simulate(model, IDENT, poses)
    rep = oracle.certify(sc2, model, IDENT, poses, got, want)
    assert rep["unexcused"] == 0, rep
    # the refitted tree keeps the original topology and carries the new boxes
    g = m.export()
    assert np.array_equal(g["links"], links)
    if builder == "lbvh":
        c = oracle.CanonicalLbvh(sc.vertices, sc.faces).export()
        assert np.array_equal(g["links"], c["links"])


def test_corrupt_tree_reports_budget_error_not_a_fault():
    """A child link bent into a cycle: every ray stops at its step budget and the map's status
    word reports RMG_ERR_TRAVERSAL_BUDGET; the context stays usable."""
    sc = scenes.box_room(seed=8, n_boxes=20)
    m = rm.Map(sc.vertices, sc.faces)
    g = m.export()
    root_links = g["links"][0]
    internal = int(root_links[0]) if root_links[0] >= 0 else int(root_links[1])
    _lib.call("rmg_map_debug_set_child", m.handle, internal, 0, 0)  # child -> root: a cycle
    model = sensors.vlp16_900()
    for cfg in [(0, 4, 8, 4), (8, 4, 8, 4), (16, 4, 8, 4, 0, 4, 2, 1)]:
        gpu_sim(m, model, scenes.room_poses(2, seed=9), attrs=("ranges",), cfg=rm.launch_config(*cfg))
        assert m.status(clear=True) == _lib.RMG_ERR_TRAVERSAL_BUDGET
    # the device is still healthy
    ok = rm.Map(sc.vertices, sc.faces)
    gpu_sim(ok, model, scenes.room_poses(1), attrs=("ranges",))
    assert ok.status() == 0


def test_corrupt_wide_tree_reports_budget_error_not_a_fault():
    """A slot of the 4-wide tree bent back to its root: the wide walk stops at its budget (or its
    stack guard) and reports RMG_ERR_TRAVERSAL_BUDGET; the binary walk of the same map is intact."""
    sc = scenes.box_room(seed=8, n_boxes=20)
    m = rm.Map(sc.vertices, sc.faces)
    model = sensors.vlp16_900()
    want = gpu_sim(m, model, scenes.room_poses(2, seed=9), attrs=("ranges",), cfg=rm.launch_config(bvh_width=2))
    _lib.call("rmg_map_debug_set_child", m.handle, 0, 2, 0)  # wide root, slot 0 -> wide root
    gpu_sim(m, model, scenes.room_poses(2, seed=9), attrs=("ranges",), cfg=rm.launch_config(bvh_width=4))
    assert m.status(clear=True) == _lib.RMG_ERR_TRAVERSAL_BUDGET
    got = gpu_sim(m, model, scenes.room_poses(2, seed=9), attrs=("ranges",), cfg=rm.launch_config(bvh_width=2))
    assert m.status() == 0 and np.array_equal(got["ranges"], want["ranges"])


def test_autotune_returns_a_config_with_identical_results():
    sc = scenes.box_room(seed=3, n_boxes=40)
    m = rm.Map(sc.vertices, sc.faces)
    model = sensors.vlp16_900()
    poses = scenes.room_poses(6, seed=4)
    want = gpu_sim(m, model, poses)
    sim = rm.make_simulator(model, m)
    cfg = sim.autotune(torch.from_numpy(poses).cuda(), attrs=ALL, reps=2)
    assert cfg.tile_w * cfg.tile_h == 32 and cfg.bvh_width in (2, 4, 8) and cfg.packet in (0, 1)
    got = gpu_sim(m, model, poses, cfg=cfg)
    for a in ALL:
        assert np.array_equal(got[a].view(np.uint8), want[a].view(np.uint8)), a


def test_stream_wait_timeout_and_success():
    lib = _lib.load()
    s = torch.cuda.Stream()
    assert lib.rmg_stream_wait(s.cuda_stream, 1000) == 0
