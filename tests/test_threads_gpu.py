"""Several host threads simulating on one map at once (the simulators' simulate is const, so
rmagine allows it): device form on one stream per thread, and the host-buffer form, whose calls
create their own streams and share the staging pool.  Every thread's results must equal the
same call made alone."""
import threading

import numpy as np
import pytest
import torch

import rmagine_gb300 as rm
from rmagine_gb300 import scenes, sensors

pytestmark = pytest.mark.gpu
N_THREADS = 4


@pytest.fixture(scope="module")
def world(built):
    torch.cuda.set_device(0)
    sc = scenes.terrain(grid=192, size=150.0, n_boxes=150, seed=61)
    m = rm.Map(sc.vertices, sc.faces)
    models = [sensors.ouster_like(rows=32, cols=512), sensors.depth_camera(128, 96), sensors.vlp16_900(),
              sensors.ouster_like(rows=16, cols=256)]
    poses = [scenes.terrain_poses(sc, 6 + 3 * i, seed=62 + i, size=150.0) for i in range(N_THREADS)]
    want = []
    for mod, p in zip(models, poses):
        res = rm.make_simulator(mod, m).simulate(torch.from_numpy(p).cuda())
        torch.cuda.synchronize()
        want.append({a: getattr(res, a).cpu() for a in rm.ATTRIBUTES})
    return m, models, poses, want


def _run_threads(fn):
    errors = []

    def wrap(i):
        try:
            fn(i)
        except Exception as e:  # reported by the main thread
            errors.append((i, e))

    ts = [threading.Thread(target=wrap, args=(i,), daemon=True) for i in range(N_THREADS)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=120)
    assert not any(t.is_alive() for t in ts), "a thread did not finish"
    assert not errors, errors


def _same(got, want):
    for a in want:
        assert torch.equal(got[a].contiguous().view(torch.uint8), want[a].contiguous().view(torch.uint8)), a


def test_device_form_from_threads_on_own_streams(world):
    m, models, poses, want = world
    got = [None] * N_THREADS

    def work(i):
        torch.cuda.set_device(0)
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            sim = rm.make_simulator(models[i], m)
            for _ in range(3):
                res = sim.simulate(torch.from_numpy(poses[i]).cuda())
            s.synchronize()
            got[i] = {a: getattr(res, a).cpu() for a in rm.ATTRIBUTES}

    _run_threads(work)
    for g, w in zip(got, want):
        _same(g, w)
    assert m.status() == 0


@pytest.mark.parametrize("pin", [True, False])
def test_host_form_from_threads(world, pin):
    m, models, poses, want = world
    got = [None] * N_THREADS

    def work(i):
        torch.cuda.set_device(0)
        sim = rm.make_simulator(models[i], m)
        W, H = sim.sensor.width, sim.sensor.height
        for _ in range(3):
            hb = rm.resize_memory_bundle(rm.IntAttrAll(), W, H, poses[i].shape[0], device="cpu", pin_memory=pin)
            sim.simulate(torch.from_numpy(poses[i]), hb)
        got[i] = {a: getattr(hb, a) for a in rm.ATTRIBUTES}

    _run_threads(work)
    for g, w in zip(got, want):
        _same(g, w)
    assert m.status() == 0
