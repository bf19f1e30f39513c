"""Pins the oracle (CPU): the reference's own known answers, and bitwise agreement with
rmagine's code compiled from its sources (oracle/_ref) where that code builds."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from rmagine_gb300 import scenes, sensors

GOLD = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())
IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def single_ray_model():
    return sensors.OnDnModel(width=1, height=1, range=sensors.Interval(0.0, 100.0),
                             origs=np.zeros((1, 3), np.float32), dirs=np.array([[1, 0, 0]], np.float32))


MODELS = {
    "example_spherical": sensors.example_spherical,
    "example_pinhole": sensors.example_pinhole,
    "example_o1dn": sensors.example_o1dn,
    "example_ondn": sensors.example_ondn,
}


def cube_results(model, n_poses=100):
    v, f = scenes.gen_cube()
    sc = oracle.Scene(v, f)
    T = np.tile(IDENT, (n_poses, 1))
    return sc.simulate(model, IDENT, T), model


def last_scan(res, model, key):
    n = model.size()
    return res[key][99 * n:100 * n]


def test_known_answer_spherical():
    g = GOLD["spherical_cube_range"]
    res, m = cube_results(sensors.example_spherical())
    r = last_scan(res, m, "ranges")[m.getBufferId(m.phi.size // 2, 0)]
    assert abs(r - g["expect"]) <= g["tol"]


def test_known_answer_pinhole():
    g = GOLD["pinhole_cube_point"]
    res, m = cube_results(sensors.example_pinhole())
    r = last_scan(res, m, "ranges")[m.getBufferId(0, 0)]
    p = oracle.directions(m)[0] * r
    assert np.abs(p - np.array(g["expect"])).sum() <= g["tol"]


def test_known_answer_o1dn_point_normal_range():
    res, m = cube_results(sensors.example_o1dn())
    r = last_scan(res, m, "ranges")[0]
    p = np.asarray(m.orig, np.float32) + m.dirs[0] * r
    g = GOLD["o1dn_cube_point"]
    assert np.abs(p - np.array(g["expect"])).sum() <= g["tol"]
    g = GOLD["o1dn_cube_normal"]
    n = last_scan(res, m, "normals")[0]
    assert np.linalg.norm(n - np.array(g["expect"])) <= g["tol"]
    g = GOLD["o1dn_cube_range"]
    assert abs(r - g["expect"]) <= g["tol"]
    # points attribute = dir*t + orig (O1DnSimulatorEmbree.tcc:132)
    assert np.abs(last_scan(res, m, "points")[0] - p).max() < 1e-6


def test_known_answer_ondn():
    g = GOLD["ondn_single_ray_range"]
    res, m = cube_results(single_ray_model())
    assert abs(res["ranges"][0] - g["expect"]) <= g["tol"]
    g = GOLD["ondn_cube_range"]
    res, m = cube_results(sensors.example_ondn())
    assert abs(last_scan(res, m, "ranges")[0] - g["expect"]) <= g["tol"]


def test_miss_semantics():
    """SphereSimulatorEmbree.tcc:189-248: misses write range.max + 1, NaN points/normals, UINT32_MAX ids."""
    v, f = scenes.gen_cube()
    sc = oracle.Scene(v, f)
    m = sensors.example_spherical()
    T = IDENT.copy()
    T[4] = 50.0  # far outside the cube: most rays miss
    res = sc.simulate(m, IDENT, T[None])
    miss = res["hits"] == 0
    assert miss.sum() > 0
    assert np.all(res["ranges"][miss] == np.float32(101.0))
    assert np.all(np.isnan(res["points"][miss])) and np.all(np.isnan(res["normals"][miss]))
    assert np.all(res["face_ids"][miss] == 0xFFFFFFFF)


def test_hits_flag_uses_range_min():
    """hits = (t >= range.min) while ranges keeps t (SphereSimulatorEmbree.tcc:110-125)."""
    v, f = scenes.gen_cube()
    sc = oracle.Scene(v, f)
    m = sensors.example_spherical()
    m.range = sensors.Interval(0.52, 100.0)
    res = sc.simulate(m, IDENT, IDENT[None])
    near = (res["face_ids"] != 0xFFFFFFFF) & (res["ranges"] < 0.52)
    assert near.sum() > 0
    assert np.all(res["hits"][near] == 0)
    assert np.all(res["hits"][(res["ranges"] >= 0.52) & (res["ranges"] <= 100.0)] == 1)


def test_oracle_agrees_with_fp64_on_room(tmp_path):
    """The binary32 watertight oracle against binary64 re-intersection: every ray's face is the
    true closest face except within the 1e-6 barycentric band or a t tie."""
    sc_ = scenes.box_room(seed=3, n_boxes=40)
    sc = oracle.Scene(sc_.vertices, sc_.faces)
    m = sensors.vlp16_900()
    T = scenes.room_poses(2, seed=4)
    res = sc.simulate(m, IDENT, T, attrs=("ranges", "face_ids", "hits"))
    rng = np.random.default_rng(0)
    gids = rng.choice(res["ranges"].size, 3000, replace=False).astype(np.uint64)
    o, d = sc.rays(m, IDENT, T, gids)
    bad = 0
    for j, g in enumerate(gids):
        fc = int(res["face_ids"][g])
        if fc == 0xFFFFFFFF:
            continue
        hit, t, b = sc.intersect_f64(o[j], d[j], fc)
        assert hit
        if abs(t - res["ranges"][g]) > 1e-4 * max(1.0, t) and abs(b) > 1e-6:
            bad += 1
    assert bad == 0


# ---- pins against the reference compiled from its own sources ----------------
def test_presets_match_reference(ref_lib):
    for i, fn in enumerate([sensors.vlp16_900, sensors.vlp16_360, sensors.example_spherical]):
        out = np.zeros(8, np.float32)
        ref_lib.ref_preset_spherical(i, _p(out))
        m = fn()
        mine = np.array([m.phi.min, m.phi.inc, m.phi.size, m.theta.min, m.theta.inc, m.theta.size, m.range.min,
                         m.range.max], np.float32)
        assert np.array_equal(out, mine), fn.__name__
    out = np.zeros(8, np.float32)
    ref_lib.ref_preset_pinhole(_p(out))
    m = sensors.example_pinhole()
    assert np.array_equal(out, np.array([m.width, m.height, m.range.min, m.range.max, *m.f, *m.c], np.float32))
    d = np.zeros((200, 3), np.float32)
    o = np.zeros(3, np.float32)
    r = np.zeros(2, np.float32)
    ref_lib.ref_example_o1dn(_p(d), _p(o), _p(r))
    assert np.array_equal(d, sensors.example_o1dn().dirs)
    og = np.zeros((200, 3), np.float32)
    ref_lib.ref_example_ondn(_p(og), _p(d), _p(r))
    assert np.array_equal(og, sensors.example_ondn().origs) and np.array_equal(d, sensors.example_ondn().dirs)


@pytest.mark.parametrize("model", ["vlp16_900", "ouster_like", "example_spherical", "example_pinhole",
                                   "depth_camera"])
def test_oracle_directions_match_reference(ref_lib, model):
    m = getattr(sensors, model)()
    ref = np.zeros((m.size(), 3), np.float32)
    if isinstance(m, sensors.SphericalModel):
        ref_lib.ref_dirs_spherical(C.c_float(m.phi.min), C.c_float(m.phi.inc), C.c_uint32(m.phi.size),
                                   C.c_float(m.theta.min), C.c_float(m.theta.inc), C.c_uint32(m.theta.size), _p(ref))
    else:
        ref_lib.ref_dirs_pinhole(C.c_uint32(m.width), C.c_uint32(m.height), C.c_float(m.f[0]), C.c_float(m.f[1]),
                                 C.c_float(m.c[0]), C.c_float(m.c[1]), _p(ref))
    assert np.array_equal(ref, oracle.directions(m))


def test_oracle_rays_match_reference_pose_math(ref_lib):
    """Tsm = Tbm * Tsb, d = Tsm.R * dir_s, o = Tsm.t (or Tsm * orig_s), against the reference's code."""
    rng = np.random.default_rng(5)
    n = 64
    Tbm = np.zeros((n, 8), np.float32)
    Tbm[:, :4] = scenes.random_quats(n, rng)
    Tbm[:, 4:7] = rng.uniform(-20, 20, (n, 3))
    Tsb = np.zeros(8, np.float32)
    Tsb[:4] = scenes.random_quats(1, rng)[0]
    Tsb[4:7] = [0.1, -0.2, 0.3]
    for m in (sensors.vlp16_900(), sensors.example_o1dn(), sensors.example_ondn()):
        W, H = oracle.model_size(m)
        gids = rng.choice(n * W * H, 500, replace=False).astype(np.uint64)
        sc = oracle.Scene(*scenes.gen_cube())
        o, d = sc.rays(m, Tsb, Tbm, gids)
        pid = (gids // (W * H)).astype(np.int64)
        loc = (gids % (W * H)).astype(np.int64)
        Tsm = np.zeros((gids.size, 8), np.float32)
        ref_lib.ref_transform_mult(_p(np.ascontiguousarray(Tbm[pid])), _p(np.tile(Tsb, (gids.size, 1))), _p(Tsm),
                                   C.c_uint32(gids.size))
        dirs = np.ascontiguousarray(oracle.directions(m)[loc])
        dref = np.zeros_like(dirs)
        ref_lib.ref_quat_rotate(_p(np.ascontiguousarray(Tsm[:, :4])), _p(dirs), _p(dref), C.c_uint32(gids.size))
        assert np.array_equal(d, dref)
        if isinstance(m, sensors.SphericalModel):
            oref = Tsm[:, 4:7]
        else:
            so = np.tile(np.asarray(m.orig, np.float32), (gids.size, 1)) if isinstance(m, sensors.O1DnModel) \
                else np.ascontiguousarray(m.origs[loc])
            oref = np.zeros_like(so)
            ref_lib.ref_transform_point(_p(Tsm), _p(np.ascontiguousarray(so)), _p(oref), C.c_uint32(gids.size))
        assert np.array_equal(o, oref)


def test_euler_matches_reference(ref_lib):
    rng = np.random.default_rng(6)
    rpy = rng.uniform(-3.1, 3.1, (100, 3)).astype(np.float32)
    ref = np.zeros((100, 4), np.float32)
    ref_lib.ref_euler_to_quat(_p(rpy), _p(ref), C.c_uint32(100))
    mine = scenes.euler_to_quat(rpy[:, 0], rpy[:, 1], rpy[:, 2])
    assert np.array_equal(ref, mine)
