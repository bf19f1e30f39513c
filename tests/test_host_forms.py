"""Host forms of the simulators: rmg_simulate_host and rmg_simulate_scene_host (the Embree
simulators' RAM bundles, SphereSimulatorEmbree.hpp:130-155) against the device forms.

Bar: every attribute bit-identical to the device form, for pinned and pageable destinations,
for every chunking of the poses (one pose per chunk up to one chunk for all), for any subset of
attributes, and through a tuned launch configuration.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import rmagine_gb300 as rm
from rmagine_gb300 import _lib, scenes, sensors

ALL = rm.ATTRIBUTES
IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)


def test_null_arguments_are_rejected_before_any_device_work(built):
    lib = _lib.load()
    T = _lib.TransformC()
    out = _lib.OutputsC()
    assert lib.rmg_simulate_host(None, None, C.byref(T), None, 1, C.byref(out), None, None) == _lib.RMG_ERR_INVALID_ARG
    assert lib.rmg_simulate_scene_host(None, None, C.byref(T), None, 1, C.byref(out), None) == \
        _lib.RMG_ERR_INVALID_ARG
    assert lib.rmg_host_set_pipeline(0, 0) == _lib.RMG_OK
    assert lib.rmg_host_set_pipeline(0, 4) == _lib.RMG_ERR_UNSUPPORTED


def _device(sim, poses, attrs):
    res = sim.simulate(torch.from_numpy(poses).cuda(), attrs=attrs)
    torch.cuda.synchronize()
    return {a: getattr(res, a).cpu() for a in attrs}


def _host(sim, poses, attrs, pin):
    W, H = sim.sensor.width, sim.sensor.height
    hb = rm.resize_memory_bundle(rm.Bundle(*attrs), W, H, poses.shape[0], device="cpu", pin_memory=pin)
    for a in attrs:  # a pattern the results must overwrite
        getattr(hb, a).view(torch.uint8).fill_(0xA5)
    sim.simulate(torch.from_numpy(poses), hb)
    return {a: getattr(hb, a) for a in attrs}


def _same(got, want):
    for a in want:
        g, w = got[a].contiguous().view(torch.uint8), want[a].contiguous().view(torch.uint8)
        assert torch.equal(g, w), a


@pytest.fixture
def chunk_bytes():
    yield lambda b, streams=0: _lib.call("rmg_host_set_pipeline", int(b), int(streams))
    _lib.call("rmg_host_set_pipeline", 0, 0)


@pytest.mark.gpu
@pytest.mark.parametrize("pin", [True, False])
@pytest.mark.parametrize("streams", [1, 2, 3])
@pytest.mark.parametrize("chunk", [1, 3 * 900 * 16 * 33, 0])
def test_host_form_equals_device_form(built, chunk_bytes, pin, streams, chunk):
    """chunk 1: one pose per chunk (7 chunks through 4 staging slots); 3 poses of all seven
    attributes per chunk: a ragged last chunk; 0: the default, one chunk of 4 and one of 3;
    each over 1, 2 or 3 compute streams."""
    sc = scenes.box_room(seed=11, n_boxes=40)
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.make_simulator(sensors.vlp16_900(), m)
    poses = scenes.room_poses(7, seed=12)
    want = _device(sim, poses, ALL)
    chunk_bytes(chunk, streams)
    _same(_host(sim, poses, ALL, pin), want)


@pytest.mark.gpu
@pytest.mark.parametrize("attrs", [("ranges",), ("hits", "normals"), ("points", "face_ids")])
def test_host_form_subsets_and_one_pose(built, chunk_bytes, attrs):
    sc = scenes.terrain(grid=96, size=60.0, n_boxes=40, seed=3)
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.make_simulator(sensors.example_pinhole(), m)
    poses = scenes.terrain_poses(sc, 5, seed=4, size=60.0)
    chunk_bytes(1)
    for n in (1, 5):
        _same(_host(sim, poses[:n].copy(), attrs, True), _device(sim, poses[:n].copy(), attrs))


@pytest.mark.gpu
def test_host_form_keeps_the_tuned_launch_config(built):
    sc = scenes.terrain(grid=128, size=80.0, n_boxes=60, seed=5)
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.make_simulator(sensors.ouster_like(rows=32, cols=256), m)
    poses = scenes.terrain_poses(sc, 9, seed=6, size=80.0)
    want = _device(sim, poses, ALL)
    sim.launch_config = rm.launch_config(packet=1)
    _same(_host(sim, poses, ALL, True), want)
    sim.launch_config = rm.launch_config(bvh_width=4, tile_w=16, tile_h=2)
    _same(_host(sim, poses, ALL, False), want)


@pytest.mark.gpu
def test_scene_host_form_equals_device_form(built, chunk_bytes):
    cube_v, cube_f = scenes.gen_cube()
    room = scenes.box_room(seed=4, n_boxes=6, half=3.0, height=2.5)
    geoms = [rm.Map(cube_v, cube_f), rm.Map(room.vertices, room.faces)]
    insts = [rm.Instance(1, IDENT, geom_id=1, object_id=7),
             rm.Instance(0, np.array([0, 0, 0, 1, 1.5, 0.5, 1.0, 0], np.float32), (0.4, 0.4, 0.4), 2, 9),
             rm.Instance(0, np.array([0, 0, 0.3826834, 0.9238795, -1.0, -1.2, 0.8, 0], np.float32), (0.3, 0.6, 0.3),
                         3, 11)]
    scene = rm.Scene(geoms, insts)
    sim = rm.make_simulator(sensors.vlp16_900(), scene)
    poses = scenes.room_poses(5, seed=8, half=2.0)
    want = _device(sim, poses, ALL)
    for chunk, streams in ((1, 3), (1, 1), (0, 0)):
        chunk_bytes(chunk, streams)
        for pin in (True, False):
            _same(_host(sim, poses, ALL, pin), want)



@pytest.mark.gpu
def test_host_form_o1dn_ondn_and_a_huge_range_max(built, chunk_bytes):
    """Points of large host-form calls are formed on the host from the ranges (with the sensor origin
    for O1Dn / OnDn, above 64 MB of points); they must equal the device form bit for bit, with a
    sensor offset, every chunking, pinned and pageable, and for a range.max so large that
    range.max + 1 rounds to range.max (then the points are copied from the device instead)."""
    sc = scenes.terrain(grid=80, size=50.0, n_boxes=30, seed=13)
    m = rm.Map(sc.vertices, sc.faces)
    rng = np.random.default_rng(14)
    models = [sensors.O1DnModel(width=5000, height=20, range=sensors.Interval(0.5, 40.0), orig=(0.1, -0.2, 0.3),
                                dirs=sensors.sphere_directions(100000, seed=15)),
              sensors.OnDnModel(width=400, height=250, range=sensors.Interval(0.0, 130.0),
                                origs=rng.uniform(-0.5, 0.5, (100000, 3)).astype(np.float32),
                                dirs=sensors.sphere_directions(100000, seed=16)),
              sensors.ouster_like(128, 800, 45.0, 0.5, 3.0e7)]
    poses = scenes.terrain_poses(sc, 60, seed=17, size=50.0)  # 6 M rays, 72 MB of points
    for model in models:
        sim = rm.make_simulator(model, m)
        sim.setTsb(np.array([0, 0, np.sin(0.2), np.cos(0.2), 0.05, 0.0, 0.1, 0], np.float32))
        want = _device(sim, poses, ALL)
        for chunk, streams in ((8 << 20, 2), (0, 0)):
            chunk_bytes(chunk, streams)
            for policy in (0, 1):  # points formed on the host, points copied
                _lib.call("rmg_host_set_points_policy", policy)
                for pin in (True, False):
                    _same(_host(sim, poses, ALL, pin), want)
                    sub = ("ranges", "points")
                    _same(_host(sim, poses, sub, pin), {a: want[a] for a in sub})
        _lib.call("rmg_host_set_points_policy", 0)
        del want
