"""O1Dn / OnDn tables of scattered directions are visited in a sorted order (rmg_sensor_create),
while every per-ray input and output keeps the table's own order: the outputs equal those of the
same rays given in the sorted order, permuted back, bit for bit, and the oracle's; pose gradients
agree to float accumulation order."""
import numpy as np
import pytest
import torch

import oracle
import rmagine_gb300 as rm
from rmagine_gb300 import grad as rg
from rmagine_gb300 import scenes, sensors

pytestmark = pytest.mark.gpu
IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)


@pytest.fixture(scope="module")
def terrain(built):
    torch.cuda.set_device(0)
    sc = scenes.terrain(grid=128, n_boxes=80, seed=21)
    return sc, rm.Map(sc.vertices, sc.faces), scenes.terrain_poses(sc, 5, seed=22)


def outputs(m, model, poses, attrs=rm.ATTRIBUTES):
    sim = rm.make_simulator(model, m)
    res = sim.simulate(torch.from_numpy(np.ascontiguousarray(poses, np.float32)).cuda(), attrs=attrs)
    torch.cuda.synchronize()
    out = {}
    for a in attrs:
        t = getattr(res, a).cpu().numpy()
        out[a] = t.view(np.uint32) if a.endswith("_ids") else t
    return sim, out


def test_scattered_o1dn_table_is_sorted_and_outputs_keep_the_table_order(terrain):
    sc, m, poses = terrain
    dirs = sensors.sphere_directions(4000, seed=23)
    scattered = sensors.O1DnModel(width=4000, height=1, range=sensors.Interval(0.3, 130.0), orig=(0.1, 0.0, 0.2),
                                  dirs=dirs)
    sim, got = outputs(m, scattered, poses)
    order = sim.sensor.visit_order()
    assert order is not None and np.array_equal(np.sort(order), np.arange(4000))
    presorted = sensors.O1DnModel(width=4000, height=1, range=scattered.range, orig=scattered.orig,
                                  dirs=np.ascontiguousarray(dirs[order]))
    sim2, want = outputs(m, presorted, poses)
    assert sim2.sensor.visit_order() is None  # already coherent: visited as given
    P = poses.shape[0]
    for a in got:
        g = got[a].reshape(P, 4000, -1)[:, order]
        assert np.array_equal(g.view(np.uint8), want[a].reshape(P, 4000, -1).view(np.uint8)), a
    ocs = oracle.Scene(sc.vertices, sc.faces)
    ref = ocs.simulate(scattered, IDENT, poses)
    rep = oracle.certify(ocs, scattered, IDENT, poses, {a: got[a].reshape(ref[a].shape) for a in got}, ref)
    assert rep["unexcused"] == 0, rep


def test_scattered_ondn_table(terrain):
    sc, m, poses = terrain
    rng = np.random.default_rng(24)
    dirs = sensors.sphere_directions(2000, seed=25)
    origs = rng.uniform(-0.3, 0.3, (2000, 3)).astype(np.float32)
    model = sensors.OnDnModel(width=40, height=50, range=sensors.Interval(0.0, 130.0), origs=origs, dirs=dirs)
    sim, got = outputs(m, model, poses)
    order = sim.sensor.visit_order()
    assert order is not None
    ocs = oracle.Scene(sc.vertices, sc.faces)
    ref = ocs.simulate(model, IDENT, poses)
    rep = oracle.certify(ocs, model, IDENT, poses, {a: got[a].reshape(ref[a].shape) for a in got}, ref)
    assert rep["unexcused"] == 0, rep


def test_coherent_tables_keep_their_order(built):
    torch.cuda.set_device(0)
    beams = sensors.ouster_like(32, 256)
    table = rm.make_simulator(beams, rm.Map(*scenes.gen_cube())).sensor.directions()
    for model in (sensors.example_o1dn(), sensors.example_ondn(),
                  sensors.O1DnModel(width=256, height=32, range=sensors.Interval(0.0, 100.0), orig=(0, 0, 0),
                                    dirs=table)):
        assert rm.make_simulator(model, rm.Map(*scenes.gen_cube())).sensor.visit_order() is None


def test_pose_gradient_over_a_sorted_table(terrain):
    sc, m, poses = terrain
    dirs = sensors.sphere_directions(3000, seed=26)
    est = scenes.perturb_poses(poses, 27, 0.1, 2.0)
    grads = []
    for d in (dirs, None):
        if d is None:
            d = np.ascontiguousarray(dirs[order])
        model = sensors.O1DnModel(width=3000, height=1, range=sensors.Interval(0.3, 130.0), orig=(0.0, 0.0, 0.1),
                                  dirs=d)
        sim = rm.make_simulator(model, m)
        if d is dirs:
            order = sim.sensor.visit_order()
            assert order is not None
        obs = sim.simulate(torch.from_numpy(poses).cuda(), attrs=("ranges",)).ranges
        g, loss = rg.range_pose_grad(sim, torch.from_numpy(est).cuda(), obs, 0.2)
        grads.append((g.cpu().numpy(), loss.cpu().numpy()))
    (g0, l0), (g1, l1) = grads
    np.testing.assert_allclose(g0, g1, rtol=1e-4, atol=1e-4 * np.abs(g1).max())
    np.testing.assert_allclose(l0, l1, rtol=1e-5)


def test_tiles_fit_one_row_and_one_column_tables(terrain):
    sc, m, poses = terrain
    dirs = sensors.sphere_directions(640, seed=28)
    for W, H in ((640, 1), (1, 640), (2, 320)):
        model = sensors.O1DnModel(width=W, height=H, range=sensors.Interval(0.3, 130.0), orig=(0.0, 0.0, 0.1),
                                  dirs=dirs)
        _, base = outputs(m, model, poses)
        for cfg in (rm.launch_config(16, 4, 8, 4, bvh_width=2, packet=0), rm.launch_config(16, 4, 32, 1, packet=0),
                    rm.launch_config(16, 4, 1, 32, packet=0), rm.launch_config(16, 4, 8, 4, packet=1)):
            sim = rm.make_simulator(model, m)
            sim.launch_config = cfg
            res = sim.simulate(torch.from_numpy(poses).cuda(), attrs=rm.ATTRIBUTES)
            for a in rm.ATTRIBUTES:
                assert np.array_equal(getattr(res, a).cpu().numpy().view(np.uint8), base[a].view(np.uint8)), (W, H, a)


def test_sorted_table_with_zero_and_nan_directions(terrain):
    sc, m, poses = terrain
    dirs = sensors.sphere_directions(1200, seed=29)
    dirs[5::97] = 0.0
    dirs[11::89] = np.nan
    model = sensors.O1DnModel(width=1200, height=1, range=sensors.Interval(0.3, 130.0), orig=(0.0, 0.0, 0.1),
                              dirs=dirs)
    sim, got = outputs(m, model, poses)
    order = sim.sensor.visit_order()
    assert order is not None and np.array_equal(np.sort(order), np.arange(1200))
    bad = np.nonzero(~np.isfinite(dirs).all(1) | (np.abs(dirs).sum(1) == 0))[0]
    assert set(order[-bad.size:].tolist()) == set(bad.tolist())  # visited last
    ocs = oracle.Scene(sc.vertices, sc.faces)
    ref = ocs.simulate(model, IDENT, poses)
    rep = oracle.certify(ocs, model, IDENT, poses, {a: got[a].reshape(ref[a].shape) for a in got}, ref)
    assert rep["unexcused"] == 0, rep
    P = poses.shape[0]
    assert np.all(got["hits"].reshape(P, -1)[:, bad] == 0)
