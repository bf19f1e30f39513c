"""Fused simulate -> statistics -> Umeyama (rmg_simulate_statistics) and the device correction loop.

The fused launch must equal rmagine's two-step inner loop (tests/embree/correction_rcc.cpp:139-160:
simulate the model at the estimate, then statistics_p2l / _p2p against the dataset scan):
n_meas exactly and the means / covariance to binary32 rounding, against both the GPU's own
simulate + statistics pair and the binary64 oracle.  The correction loop built from it must
converge like the reference's RCC test (|dz|, |dyaw| < 1e-3)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from oracle import stats as ost
from rmagine_gb300 import scenes, sensors, transforms

from test_rcc import converged, rcc_model, start_pose

IDENT = transforms.identity()


# ---- CPU ---------------------------------------------------------------------------------
def test_oracle_fused_step_is_identity_at_the_true_pose():
    """At the pose the dataset scan was taken from, every hit pairs with itself: the statistics
    have equal means, n = number of hits, and Umeyama returns the identity."""
    v, f = scenes.gen_cube()
    sc = oracle.Scene(v, f)
    model = rcc_model()
    data = sc.simulate(model, IDENT, IDENT[None], attrs=("hits", "points"))
    for p2l in (True, False):
        st, R, t, q, ok = ost.simulate_statistics(sc, model, IDENT, IDENT[None], data["points"],
                                                  dmask=data["hits"], point_to_plane=p2l)
        assert st["n"][0] == int(data["hits"].sum()) > 0
        assert np.abs(st["dataset_mean"] - st["model_mean"]).max() < 1e-6
        assert np.abs(R[0] - np.eye(3)).max() < 1e-9 and np.abs(t).max() < 1e-9


def test_oracle_fused_step_reduces_the_pose_error():
    """One inner step from the RCC test's start pose moves the estimate towards the truth in both
    the height and the yaw that the start pose perturbs."""
    v, f = scenes.gen_cube()
    sc = oracle.Scene(v, f)
    model = rcc_model()
    data = sc.simulate(model, IDENT, IDENT[None], attrs=("hits", "points"))
    T0 = start_pose()
    st, R, t, q, ok = ost.simulate_statistics(sc, model, IDENT, T0[None], data["points"], dmask=data["hits"],
                                              max_dist=100.0)
    Tn = IDENT.copy()
    Tn[:4] = q[0]
    Tn[4:7] = t[0]
    T1 = transforms.compose(T0, Tn)
    for err in (lambda T: abs(float(T[6])), lambda T: abs(float(transforms.yaw(T[:4])))):
        assert err(T1) < 0.95 * err(T0)


def test_entry_points_reject_bad_arguments_without_a_gpu(built):
    from rmagine_gb300 import _lib

    lib = _lib.load()
    pc = _lib.ConstraintsC(1.0, 0, 0)
    scan = _lib.ScanC(None, None, None, 0)
    T = _lib.TransformC()
    assert lib.rmg_simulate_statistics(None, None, None, None, 1, None, None, 0, None, 1, None, None,
                                       None) == _lib.RMG_ERR_INVALID_ARG
    assert lib.rmg_simulate_statistics(C.c_void_p(1), C.c_void_p(1), C.byref(T), None, 1, C.byref(scan), None, 0,
                                       C.byref(pc), 1, None, None, None) == _lib.RMG_ERR_INVALID_ARG
    assert lib.rmg_transforms_compose(None, 0, None, 0, None, 1, None) == _lib.RMG_ERR_INVALID_ARG
    assert lib.rmg_transforms_compose(None, 0, None, 0, None, 0, None) == _lib.RMG_OK


# ---- GPU ---------------------------------------------------------------------------------
def _models():
    rng = np.random.default_rng(7)
    d = rng.standard_normal((2000, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = rng.uniform(-0.05, 0.05, (2000, 3)).astype(np.float32)
    return {
        "spherical": sensors.vlp16_900(),
        "pinhole": sensors.depth_camera(160, 120),
        "o1dn": sensors.O1DnModel(width=2000, height=1, range=sensors.Interval(0.3, 60.0),
                                  orig=(0.1, 0.0, 0.2), dirs=d),
        "ondn": sensors.OnDnModel(width=1000, height=2, range=sensors.Interval(0.3, 60.0), origs=o, dirs=d),
    }


def _room_problem(kind, n=6, seed=3):
    import torch

    import rmagine_gb300 as rm

    sc = scenes.box_room(seed=seed, n_boxes=40)
    model = _models()[kind]
    true = scenes.room_poses(n, seed=seed + 1)
    est = scenes.perturb_poses(true, seed + 2, sigma_t=0.1, sigma_r_deg=2.0)
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.make_simulator(model, m)
    data = sim.simulate(torch.from_numpy(true).cuda(), attrs=("hits", "points"))
    pre = scenes.perturb_poses(np.tile(IDENT, (n, 1)), seed + 6, sigma_t=0.02, sigma_r_deg=0.5)
    return sc, model, m, sim, true, est, data, pre


def _unfused(sim, est, data, pre, params, p2l, n):
    import torch

    from rmagine_gb300 import statistics as rs

    W, H = sim.sensor.width, sim.sensor.height
    mod = sim.simulate(torch.from_numpy(est).cuda(), attrs=("hits", "points", "normals"))
    kw = dict(pre=pre, params=params, dataset_mask=data.hits.reshape(n, W * H), model_mask=mod.hits.reshape(n, W * H))
    if p2l:
        return rs.statistics_p2l(data.points.reshape(n, W * H, 3), mod.points.reshape(n, W * H, 3),
                                 mod.normals.reshape(n, W * H, 3), **kw)
    return rs.statistics_p2p(data.points.reshape(n, W * H, 3), mod.points.reshape(n, W * H, 3), **kw)


def _close_stats(a, b, rtol):
    from rmagine_gb300 import statistics as rs

    A, B = rs.decode_stats(a), rs.decode_stats(b)
    assert np.array_equal(A["n"], B["n"]), (A["n"], B["n"])
    for k in ("dataset_mean", "model_mean", "covariance"):
        scale = 1.0 + np.abs(B[k]).max()
        assert np.abs(A[k] - B[k]).max() <= rtol * scale, (k, np.abs(A[k] - B[k]).max())


def _rot_err(qa, qb):
    return ost.rotation_angle(ost.quat_to_rot(np.reshape(qa, (-1, 4))), ost.quat_to_rot(np.reshape(qb, (-1, 4))))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["spherical", "pinhole", "o1dn", "ondn"])
@pytest.mark.parametrize("p2l", [True, False])
def test_fused_equals_simulate_then_statistics(built, kind, p2l):
    import torch

    from rmagine_gb300 import statistics as rs

    torch.cuda.set_device(0)
    n = 6
    sc, model, m, sim, true, est, data, pre = _room_problem(kind, n)
    W, H = sim.sensor.width, sim.sensor.height
    params = rs.UmeyamaReductionConstraints(max_dist=0.5 if p2l else 1.0)
    su, Tu = _unfused(sim, est, data, pre, params, p2l, n)
    sf, Tf = sim.simulate_statistics(torch.from_numpy(est).cuda(), data.points.reshape(n, W * H, 3),
                                     dataset_mask=data.hits.reshape(n, W * H), pre=pre, params=params,
                                     point_to_plane=p2l)
    torch.cuda.synchronize()
    assert m.status() == 0
    assert rs.decode_stats(sf)["n"].sum() > 0
    _close_stats(sf, su, 2e-6)
    Tf_, Tu_ = Tf.cpu().numpy(), Tu.cpu().numpy()
    assert _rot_err(Tf_[:, :4], Tu_[:, :4]).max() < 2e-5
    assert np.abs(Tf_[:, 4:7] - Tu_[:, 4:7]).max() < 2e-5


@pytest.mark.gpu
@pytest.mark.parametrize("p2l", [True, False])
def test_fused_against_the_binary64_oracle(built, p2l):
    import torch

    from rmagine_gb300 import statistics as rs

    torch.cuda.set_device(0)
    n = 6
    sc, model, m, sim, true, est, data, pre = _room_problem("spherical", n, seed=11)
    W, H = sim.sensor.width, sim.sensor.height
    max_dist = 0.5 if p2l else 1.0
    sf, Tf = sim.simulate_statistics(torch.from_numpy(est).cuda(), data.points.reshape(n, W * H, 3),
                                     dataset_mask=data.hits.reshape(n, W * H), pre=pre,
                                     params=rs.UmeyamaReductionConstraints(max_dist=max_dist), point_to_plane=p2l)
    osc = oracle.Scene(sc.vertices, sc.faces)
    st, R, t, q, ok = ost.simulate_statistics(osc, model, IDENT, est, data.points.cpu().numpy().reshape(n, -1, 3),
                                              dmask=data.hits.cpu().numpy(), pre=pre, max_dist=max_dist,
                                              point_to_plane=p2l)
    # model rays on which the GPU and the oracle may disagree (edge / tie hits, certified)
    got = sim.simulate(torch.from_numpy(est).cuda(), attrs=("hits", "ranges", "face_ids"))
    got = {"hits": got.hits.cpu().numpy(), "ranges": got.ranges.cpu().numpy(),
           "face_ids": got.face_ids.cpu().numpy().view(np.uint32)}
    want = osc.simulate(model, IDENT, est, attrs=("hits", "ranges", "face_ids"))
    rep = oracle.certify(osc, model, IDENT, est, got, want)
    assert not rep["unexcused"], rep
    G = rs.decode_stats(sf)
    assert np.abs(G["n"] - st["n"]).max() <= rep["disputed"]
    if rep["disputed"] == 0:
        for k in ("dataset_mean", "model_mean", "covariance"):
            assert np.abs(G[k] - st[k]).max() <= 1e-5 * (1.0 + np.abs(st[k]).max()), k
        T = Tf.cpu().numpy()
        assert _rot_err(T[:, :4], q).max() < 1e-4
        assert np.abs(T[:, 4:7] - t).max() < 1e-4


@pytest.mark.gpu
def test_shared_scan_and_pre_transform_equal_their_replicas_bitwise(built):
    """per_pose = 0 (one scan for every pose) and one shared pre-transform give exactly the
    results of the same data replicated per pose."""
    import torch

    import rmagine_gb300 as rm
    from rmagine_gb300 import statistics as rs

    torch.cuda.set_device(0)
    sc = scenes.box_room(seed=5, n_boxes=30)
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.SphereSimulator(m)
    sim.setModel(sensors.vlp16_900())
    W, H = sim.sensor.width, sim.sensor.height
    true = scenes.room_poses(1, seed=9)
    hyp = scenes.perturb_poses(np.tile(true, (16, 1)), 4, sigma_t=0.2, sigma_r_deg=3.0)
    data = sim.simulate(torch.from_numpy(true).cuda(), attrs=("hits", "points"))
    pre = scenes.perturb_poses(IDENT[None], 8, sigma_t=0.05, sigma_r_deg=1.0)
    P = rs.UmeyamaReductionConstraints(max_dist=1.0)
    Hd = torch.from_numpy(hyp).cuda()
    s1, T1 = sim.simulate_statistics(Hd, data.points, dataset_mask=data.hits, pre=pre, params=P)
    s2, T2 = sim.simulate_statistics(Hd, data.points.reshape(1, W * H, 3).repeat(16, 1, 1),
                                     dataset_mask=data.hits.reshape(1, -1).repeat(16, 1),
                                     pre=np.tile(pre, (16, 1)), params=P)
    assert torch.equal(s1, s2) and torch.equal(T1, T2)
    # determinism: the same call twice gives the same bits
    s3, T3 = sim.simulate_statistics(Hd, data.points, dataset_mask=data.hits, pre=pre, params=P)
    assert torch.equal(s1, s3) and torch.equal(T1, T3)


@pytest.mark.gpu
def test_dataset_ids_masks_and_empty_sets(built):
    import torch

    from rmagine_gb300 import statistics as rs

    torch.cuda.set_device(0)
    n = 4
    sc, model, m, sim, true, est, data, pre = _room_problem("spherical", n, seed=21)
    W, H = sim.sensor.width, sim.sensor.height
    rng = np.random.default_rng(0)
    ids = rng.integers(0, 3, n * W * H).astype(np.uint32)
    P = rs.UmeyamaReductionConstraints(max_dist=0.5, dataset_id=1)
    Ed = torch.from_numpy(est).cuda()
    sf, Tf = sim.simulate_statistics(Ed, data.points.reshape(n, W * H, 3), dataset_mask=data.hits.reshape(n, -1),
                                     dataset_ids=ids.reshape(n, -1), pre=pre, params=P)
    mod = sim.simulate(Ed, attrs=("hits", "points", "normals"))
    su, _ = rs.statistics_p2l(data.points.reshape(n, W * H, 3), mod.points.reshape(n, W * H, 3),
                              mod.normals.reshape(n, W * H, 3), pre=pre, params=P,
                              dataset_mask=data.hits.reshape(n, -1), model_mask=mod.hits.reshape(n, -1),
                              dataset_ids=ids.reshape(n, -1))
    _close_stats(sf, su, 2e-6)
    # nothing valid: n = 0, zero statistics, identity transform
    zero = torch.zeros(n * W * H, dtype=torch.uint8, device="cuda")
    s0, T0 = sim.simulate_statistics(Ed, data.points.reshape(n, W * H, 3), dataset_mask=zero.reshape(n, -1))
    assert rs.decode_stats(s0)["n"].max() == 0
    assert torch.equal(T0.cpu(), torch.from_numpy(np.tile(IDENT, (n, 1))))
    # zero poses: nothing to do
    e = torch.empty((0, 8), dtype=torch.float32, device="cuda")
    s, T = sim.simulate_statistics(e, data.points.reshape(n, W * H, 3)[0])
    assert s.shape == (0, 16) and T.shape == (0, 8)
    torch.cuda.synchronize()
    assert m.status() == 0


@pytest.mark.gpu
def test_compose_matches_the_host_transform_arithmetic(built):
    import torch

    from rmagine_gb300 import correction

    torch.cuda.set_device(0)
    a = scenes.perturb_poses(np.tile(IDENT, (257, 1)), 1, sigma_t=3.0, sigma_r_deg=60.0)
    b = scenes.perturb_poses(np.tile(IDENT, (257, 1)), 2, sigma_t=3.0, sigma_r_deg=60.0)
    ad, bd = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    got = correction.compose(ad, bd).cpu().numpy()
    want = transforms.compose(a, b)
    assert np.array_equal(got[:, :7], want[:, :7])
    got1 = correction.compose(ad[:1].contiguous(), bd).cpu().numpy()
    assert np.array_equal(got1[:, :7], transforms.compose(a[:1], b)[:, :7])
    correction.compose(ad, bd, out=ad)  # in place (multInplace)
    assert np.array_equal(ad.cpu().numpy()[:, :7], want[:, :7])


@pytest.mark.gpu
def test_rcc_correction_with_fused_steps_converges(built):
    """rmagine's RCC correction test (correction_rcc.cpp:60-180) run entirely on the device."""
    import torch

    import rmagine_gb300 as rm
    from rmagine_gb300 import correction
    from rmagine_gb300 import statistics as rs

    torch.cuda.set_device(0)
    v, f = scenes.gen_cube()
    m = rm.Map(v, f)
    sim = rm.SphereSimulator(m)
    sim.setModel(rcc_model())
    data = sim.simulate(torch.from_numpy(IDENT[None].copy()).cuda(), attrs=("hits", "points"))
    T = correction.correct_rcc(sim, data.points, start_pose(), dataset_mask=data.hits, n_outer=10, n_inner=5,
                               params=rs.UmeyamaReductionConstraints(max_dist=100.0))
    assert converged(T.cpu().numpy()[0]), T


@pytest.mark.gpu
def test_batched_correction_matches_the_two_step_loop(built):
    """MICP-style batch: 24 pose hypotheses around each of 2 true poses in the box room, each
    corrected against its own scan; the fused loop and the two-step loop (simulate +
    statistics_p2l) end at the same poses, closer to the truth than they started."""
    import torch

    import rmagine_gb300 as rm
    from rmagine_gb300 import correction
    from rmagine_gb300 import statistics as rs

    torch.cuda.set_device(0)
    sc = scenes.box_room(seed=2, n_boxes=60)
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.SphereSimulator(m)
    sim.setModel(sensors.vlp16_900())
    W, H = sim.sensor.width, sim.sensor.height
    true = np.repeat(scenes.room_poses(2, seed=3), 24, axis=0)
    est0 = scenes.perturb_poses(true, 5, sigma_t=0.15, sigma_r_deg=3.0)
    n = true.shape[0]
    data = sim.simulate(torch.from_numpy(true).cuda(), attrs=("hits", "points"))
    P = rs.UmeyamaReductionConstraints(max_dist=0.5)
    dp, dm = data.points.reshape(n, W * H, 3), data.hits.reshape(n, W * H)
    fused = correction.correct_rcc(sim, dp, est0, dataset_mask=dm, n_outer=6, n_inner=2, params=P).cpu().numpy()
    # the same loop with the model bundle materialised
    est = torch.from_numpy(est0).cuda()
    for _ in range(6):
        mod = sim.simulate(est, attrs=("hits", "points", "normals"))
        Tpre = torch.from_numpy(np.tile(IDENT, (n, 1))).cuda()
        for _ in range(2):
            _, T = rs.statistics_p2l(dp, mod.points.reshape(n, W * H, 3), mod.normals.reshape(n, W * H, 3),
                                     pre=Tpre, params=P, dataset_mask=dm, model_mask=mod.hits.reshape(n, W * H))
            Tpre = correction.compose(Tpre, T)
        est = correction.compose(est, Tpre)
    twostep = est.cpu().numpy()
    assert _rot_err(fused[:, :4], twostep[:, :4]).max() < 1e-4
    assert np.abs(fused[:, 4:7] - twostep[:, 4:7]).max() < 1e-4
    e0 = np.linalg.norm(est0[:, 4:7] - true[:, 4:7], axis=1)
    e1 = np.linalg.norm(fused[:, 4:7] - true[:, 4:7], axis=1)
    assert np.median(e1) < 0.5 * np.median(e0), (np.median(e0), np.median(e1))


@pytest.mark.gpu
def test_host_scans_give_the_device_result_bitwise(built):
    """Per-pose scans in pinned host memory are uploaded in pose chunks overlapped with the fused
    launches; every pose is reduced on its own, so the statistics and transforms equal one call on
    device data bit for bit (pose counts that do and do not divide into the chunks)."""
    import torch

    from rmagine_gb300 import _lib
    from rmagine_gb300 import statistics as rs

    torch.cuda.set_device(0)
    n = 11
    sc, model, m, sim, true, est, data, pre = _room_problem("spherical", n, seed=31)
    W, H = sim.sensor.width, sim.sensor.height
    P = rs.UmeyamaReductionConstraints(max_dist=0.5)
    dp, dm = data.points.reshape(n, W * H, 3), data.hits.reshape(n, W * H)
    for k in (11, 9, 2):
        E = torch.from_numpy(est[:k].copy()).cuda()
        s0, T0 = sim.simulate_statistics(E, dp[:k], dataset_mask=dm[:k], pre=pre[:k], params=P)
        s1, T1 = sim.simulate_statistics(E, dp[:k].cpu().pin_memory(), dataset_mask=dm[:k].cpu().pin_memory(),
                                         pre=pre[:k], params=P)
        torch.cuda.synchronize()
        assert not s1.is_cuda and not T1.is_cuda  # the host form returns host results
        assert torch.equal(s0.cpu(), s1) and torch.equal(T0.cpu(), T1), k
        # host poses, a single host scan for every pose, pageable memory, a small chunk size
        _lib.call("rmg_host_set_pipeline", 1, 3)
        try:
            s2, T2 = sim.simulate_statistics(torch.from_numpy(est[:k].copy()), dp[0].cpu(), dataset_mask=dm[0].cpu(),
                                             params=P)
            s3, T3 = sim.simulate_statistics(E, dp[0], dataset_mask=dm[0], params=P)
            torch.cuda.synchronize()
            assert torch.equal(s3.cpu(), s2) and torch.equal(T3.cpu(), T2), k
            s4, T4 = sim.simulate_statistics(E, dp[:k].cpu(), dataset_mask=dm[:k].cpu(), pre=pre[:k], params=P)
            assert torch.equal(s0.cpu(), s4) and torch.equal(T0.cpu(), T4), k
        finally:
            _lib.call("rmg_host_set_pipeline", 0, 0)
    assert m.status() == 0
