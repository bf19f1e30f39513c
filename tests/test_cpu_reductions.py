"""The C++ OpenMP restatements of the timed CPU baselines equal the oracle's numpy restatements:
batched statistics (point-to-point and point-to-plane, with masks and distance filters), the
range adjoint's analytic gradient and the range noise."""
import numpy as np

import oracle
from oracle import grad as og
from oracle import noise as on
from oracle import stats as ost
from rmagine_gb300 import scenes, sensors

IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)


def test_stats_batched_equals_numpy_restatement():
    rng = np.random.default_rng(0)
    B, N = 12, 3000
    src = rng.uniform(-25, 25, (B, N, 3)).astype(np.float32)
    tgt = (src + rng.normal(0, 0.5, src.shape)).astype(np.float32)
    nrm = rng.standard_normal((B, N, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=2, keepdims=True)
    dmask = (rng.uniform(size=(B, N)) > 0.1).astype(np.uint8)
    mmask = (rng.uniform(size=(B, N)) > 0.1).astype(np.uint8)
    mmask[3] = 0  # a batch without correspondences
    for kw in (dict(), dict(max_dist=1.0), dict(normals=nrm, max_dist=0.5, dmask=dmask, mmask=mmask),
               dict(max_dist=0.8, dmask=dmask)):
        want = ost.stats(*ost.correspondences(src, tgt, **kw))
        got = oracle.stats_batched(src, tgt, **kw)
        for k in want:
            np.testing.assert_allclose(got[k], want[k], rtol=1e-12, atol=1e-12, err_msg=k)


def test_pose_grad_equals_numpy_restatement():
    sc = scenes.terrain(grid=96, n_boxes=20, seed=3)
    model = sensors.ouster_like(16, 128, 45.0, 0.5, 130.0)
    true = scenes.terrain_poses(sc, 3, seed=4)
    est = scenes.perturb_poses(true, 5, 0.1, 2.0)
    ocs = oracle.Scene(sc.vertices, sc.faces)
    obs = ocs.simulate(model, IDENT, true, attrs=("ranges",))["ranges"]
    sim = ocs.simulate(model, IDENT, est, attrs=("ranges", "face_ids"))
    W, H = model.getWidth(), model.getHeight()
    f, r = sim["face_ids"], sim["ranges"]
    valid = (f != 0xFFFFFFFF) & (r >= model.range.min) & (obs >= model.range.min) & (obs <= model.range.max)
    gid = np.nonzero(valid)[0]
    rset = og.RayFaceSet(sc.vertices, sc.faces, IDENT, est, oracle.directions(model)[gid % (W * H)],
                         np.zeros((gid.size, 3)), gid // (W * H), f[gid], obs[gid])
    g_want, l_want = rset.analytic(est.shape[0], 0.2)
    g, loss = oracle.pose_grad(ocs, model, IDENT, est, f, r, obs, 0.2)
    assert np.abs(g_want).max() > 0
    np.testing.assert_allclose(g, g_want, rtol=1e-9, atol=1e-9 * np.abs(g_want).max())
    np.testing.assert_allclose(loss, l_want, rtol=1e-12)


def test_rcc_step_equals_simulate_statistics():
    sc = scenes.terrain(grid=96, n_boxes=20, seed=6)
    model = sensors.ouster_like(16, 128, 45.0, 0.5, 130.0)
    true = scenes.terrain_poses(sc, 3, seed=7)
    est = scenes.perturb_poses(true, 8, 0.1, 2.0)
    ocs = oracle.Scene(sc.vertices, sc.faces)
    data = ocs.simulate(model, IDENT, true, attrs=("hits", "points"))
    want, R, t, q, ok = ost.simulate_statistics(ocs, model, IDENT, est, data["points"], dmask=data["hits"],
                                                max_dist=0.5)
    n, WH = est.shape[0], model.getWidth() * model.getHeight()
    sim = ocs.simulate(model, IDENT, est, attrs=("hits", "points", "normals"), fast=True)
    got = oracle.stats_batched(data["points"].reshape(n, WH, 3), sim["points"].reshape(n, WH, 3),
                               normals=sim["normals"].reshape(n, WH, 3), dmask=data["hits"], mmask=sim["hits"],
                               max_dist=0.5)
    for k in want:
        np.testing.assert_allclose(got[k], want[k], rtol=1e-12, atol=1e-12, err_msg=k)
    R2, t2, _ = ost.umeyama(got)
    np.testing.assert_allclose(R2, R, atol=1e-12)
    np.testing.assert_allclose(t2, t, atol=1e-9)


def test_noise_equals_numpy_restatement():
    rr = np.random.default_rng(1).uniform(0, 150, 200_003).astype(np.float32)
    for kind, kw in ((0, dict(stddev=0.02, mean=0.01, max_range=130.0)),
                     (1, dict(stddev=0.01, range_exp=1.3, max_range=130.0)),
                     (2, dict(hit_p=0.01, ret_p=0.5, max_range=100.0))):
        want = on.apply(kind, rr, seed=42, call=3, **kw)
        want = want[0] if isinstance(want, tuple) else want
        got = oracle.noise_apply(kind, rr, 42, 3, **kw)
        if kind == 1:  # pow() of two libraries: the last bits may differ
            np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13)
        else:
            assert np.array_equal(got, want), kind
