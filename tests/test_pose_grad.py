"""Range adjoint d(loss)/d(6-DoF pose): the binary64 host reference pinned by finite differences
(CPU), and the GPU kernel against that reference and against finite differences (GPU)."""
import numpy as np
import pytest

import oracle
from oracle import grad as og
from rmagine_gb300 import scenes, sensors, transforms

IDENT = np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float32)
DELTA = 0.2


def perturbed(poses, seed, sig_t=0.1, sig_r_deg=2.0):
    rng = np.random.default_rng(seed)
    n = poses.shape[0]
    d = np.zeros((n, 8), np.float32)
    w = rng.normal(0, np.radians(sig_r_deg), (n, 3))
    th = np.linalg.norm(w, axis=1, keepdims=True)
    d[:, :3] = (w / th * np.sin(th / 2)).astype(np.float32)
    d[:, 3] = np.cos(th[:, 0] / 2).astype(np.float32)
    out = transforms.compose(poses, d)
    out[:, 4:7] += rng.normal(0, sig_t, (n, 3)).astype(np.float32)
    return out


def problem(seed=0, n_poses=6, rows=32, cols=256):
    sc = scenes.terrain(grid=96, n_boxes=60, seed=seed, size=500.0)
    model = sensors.ouster_like(rows, cols)
    true = scenes.terrain_poses(sc, n_poses, seed=seed + 1, size=500.0)
    return sc, model, true, perturbed(true, seed + 2)


def rayset(sc, model, Tbm, faces, r_sim, r_obs):
    W, H = oracle.model_size(model)
    n = Tbm.shape[0]
    rmin, rmax = model.range.min, model.range.max
    valid = (faces != 0xFFFFFFFF) & (r_sim >= rmin) & (r_obs >= rmin) & (r_obs <= rmax)
    gid = np.nonzero(valid)[0]
    dirs = oracle.directions(model)
    return og.RayFaceSet(sc.vertices, sc.faces, IDENT, Tbm, dirs[gid % (W * H)], np.zeros((gid.size, 3)),
                         gid // (W * H), faces[gid], r_obs[gid]), n


def test_oracle_gradient_matches_finite_differences():
    sc, model, true, est = problem(seed=10, n_poses=3, rows=16, cols=128)
    ocs = oracle.Scene(sc.vertices, sc.faces)
    obs = ocs.simulate(model, IDENT, true, attrs=("ranges",))["ranges"]
    sim = ocs.simulate(model, IDENT, est, attrs=("ranges", "face_ids"))
    rset, n = rayset(sc, model, est, sim["face_ids"], sim["ranges"], obs)
    fd, an, stable = rset.finite_differences(n, DELTA, h=1e-4)
    assert stable.mean() > 0.95
    rel = np.abs(fd - an).max() / np.abs(an).max()
    assert rel < 1e-3, rel


gpu = pytest.mark.gpu


@pytest.fixture(scope="module")
def rm_mod(built):
    import torch

    import rmagine_gb300 as rm

    torch.cuda.set_device(0)
    return rm


@gpu
def test_gpu_gradient_matches_fp64_reference_and_fd(rm_mod):
    import torch

    from rmagine_gb300 import grad as rg

    rm = rm_mod
    sc, model, true, est = problem(seed=20)
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.SphereSimulator(m)
    sim.setModel(model)
    obs = sim.simulate(torch.from_numpy(true).cuda(), attrs=("ranges",)).ranges
    g, loss, rs, fs = rg.range_pose_grad(sim, torch.from_numpy(est).cuda(), obs, DELTA, want_sim=True)
    torch.cuda.synchronize()
    g, loss = g.cpu().numpy(), loss.cpu().numpy()
    rs, fs = rs.cpu().numpy(), fs.cpu().numpy().view(np.uint32)
    # the fused forward equals plain simulate
    plain = sim.simulate(torch.from_numpy(est).cuda(), attrs=("ranges", "face_ids"))
    assert np.array_equal(plain.ranges.cpu().numpy(), rs)
    assert np.array_equal(plain.face_ids.cpu().numpy().view(np.uint32), fs)
    rset, n = rayset(sc, model, est, fs, rs, obs.cpu().numpy())
    an, an_loss = rset.analytic(n, DELTA)
    rel = np.abs(g - an).max() / np.abs(an).max()
    assert rel < 1e-3, rel
    assert np.abs(loss - an_loss).max() / np.abs(an_loss).max() < 1e-3
    fd, an_s, stable = rset.finite_differences(n, DELTA, h=1e-4)
    assert stable.mean() > 0.95
    assert np.abs(fd - an_s).max() / np.abs(an_s).max() < 1e-3
    assert m.status() == 0


@gpu
def test_host_observations_give_the_device_result_bitwise(rm_mod):
    """Observed ranges in pinned host memory go through the pipelined path (pose chunks uploaded
    while the previous chunk computes); gradient, loss and the simulated ranges equal one call on
    device data bit for bit, for pose counts that do and do not divide into the chunks."""
    import torch

    from rmagine_gb300 import grad as rg

    rm = rm_mod
    sc, model, true, est = problem(seed=21, n_poses=11)
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.SphereSimulator(m)
    sim.setModel(model)
    obs = sim.simulate(torch.from_numpy(true).cuda(), attrs=("ranges",)).ranges
    for n in (11, 8, 1):
        Td = torch.from_numpy(est[:n].copy()).cuda()
        per = obs.numel() // 11
        g0, l0, r0, f0 = rg.range_pose_grad(sim, Td, obs[:n * per], DELTA, want_sim=True)
        host = obs[:n * per].cpu().pin_memory()
        g1, l1, r1, f1 = rg.range_pose_grad(sim, torch.from_numpy(est[:n].copy()).pin_memory(), host, DELTA,
                                            want_sim=True)
        torch.cuda.synchronize()
        assert not g1.is_cuda  # the host form returns host results
        for a, b in ((g0, g1), (l0, l1), (r0, r1), (f0, f1)):
            assert torch.equal(a.cpu(), b), n
        # pageable observations, device poses, one pose per chunk over three compute streams
        from rmagine_gb300 import _lib
        _lib.call("rmg_host_set_pipeline", 1, 3)
        try:
            g2, l2 = rg.range_pose_grad(sim, Td, obs[:n * per].cpu(), DELTA)
            assert torch.equal(g0.cpu(), g2) and torch.equal(l0.cpu(), l2), n
        finally:
            _lib.call("rmg_host_set_pipeline", 0, 0)
    assert m.status() == 0


@gpu
def test_gpu_gradient_on_a_plane_matches_fd_of_retraced_ranges(rm_mod):
    """Flat ground (two coplanar triangles): every ray's range is a smooth function of the pose,
    so GPU gradients compare directly with binary64 central differences of re-traced ranges."""
    import torch

    from rmagine_gb300 import grad as rg

    rm = rm_mod
    v = np.array([[-100, -100, 0], [100, -100, 0], [100, 100, 0], [-100, 100, 0]], np.float32)
    f = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    m = rm.Map(v, f)
    model = sensors.SphericalModel(phi=sensors.DiscreteInterval(-0.6, 0.02, 16),
                                   theta=sensors.DiscreteInterval(-3.1, 0.05, 124),
                                   range=sensors.Interval(0.1, 60.0))
    sim = rm.SphereSimulator(m)
    sim.setModel(model)
    true = np.tile(IDENT, (4, 1))
    true[:, 6] = [1.0, 1.5, 2.0, 2.5]
    est = perturbed(true, 3, sig_t=0.05, sig_r_deg=1.0)
    obs = sim.simulate(torch.from_numpy(true).cuda(), attrs=("ranges",)).ranges
    g, loss = rg.range_pose_grad(sim, torch.from_numpy(est).cuda(), obs, DELTA)
    torch.cuda.synchronize()
    g = g.cpu().numpy()
    # binary64 FD with the plane re-intersected for every perturbed pose
    dirs = oracle.directions(model).astype(np.float64)
    W, H = 124, 16
    obs_h = obs.cpu().numpy().reshape(4, -1)
    fd = np.zeros((4, 6))
    h = 1e-4
    for p in range(4):
        Rbm = og.quat_to_rot(est[p, :4].astype(np.float64))
        tbm = est[p, 4:7].astype(np.float64)

        def L(rho, om):
            Rw = og.rodrigues(om)
            o = Rbm @ rho + tbm
            d = dirs @ (Rbm @ Rw).T
            r = -o[2] / d[:, 2]
            ok = (r > 0) & (r <= 60.0) & (r >= 0.1) & (obs_h[p] >= 0.1) & (obs_h[p] <= 60.0)
            return (og.huber(r - obs_h[p], DELTA) * ok).sum()

        for k in range(6):
            e = np.zeros(6)
            e[k] = h
            fd[p, k] = (L(e[:3], e[3:]) - L(-e[:3], -e[3:])) / (2 * h)
    assert np.abs(g - fd).max() / np.abs(fd).max() < 1e-3


@gpu
def test_autograd_function_returns_kernel_gradient(rm_mod):
    import torch

    from rmagine_gb300 import grad as rg

    rm = rm_mod
    sc, model, true, est = problem(seed=30, n_poses=3, rows=16, cols=128)
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.SphereSimulator(m)
    sim.setModel(model)
    obs = sim.simulate(torch.from_numpy(true).cuda(), attrs=("ranges",)).ranges
    Tbm = torch.from_numpy(est).cuda()
    xi = torch.zeros((3, 6), dtype=torch.float32, requires_grad=True)
    loss = rg.RangePoseLoss.apply(xi, sim, Tbm, obs, DELTA)
    loss.sum().backward()
    g, _ = rg.range_pose_grad(sim, Tbm, obs, DELTA)
    assert torch.equal(xi.grad, g.cpu())


@gpu
@pytest.mark.parametrize("kind", ["o1dn", "ondn"])
def test_gpu_gradient_with_ray_origins_and_sensor_offset(rm_mod, kind):
    """Sensors whose rays start off the sensor origin (O1Dn: one origin, OnDn: one per ray; random
    direction tables, walked in their sorted visiting order) behind a rotated, offset Tsb: the
    kernel's gradient against the binary64 reference with the same origins."""
    import torch

    from rmagine_gb300 import grad as rg

    rm = rm_mod
    sc = scenes.terrain(grid=96, n_boxes=60, seed=40, size=500.0)
    true = scenes.terrain_poses(sc, 5, seed=41, size=500.0)
    est = perturbed(true, 42)
    rng = np.random.default_rng(43)
    dirs = sensors.sphere_directions(3000, seed=44)
    dirs[:, 2] = -np.abs(dirs[:, 2])  # looking down at the terrain
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    dirs = dirs.astype(np.float32)
    if kind == "o1dn":
        model = sensors.O1DnModel(width=3000, height=1, range=sensors.Interval(0.3, 130.0), orig=(0.2, -0.1, 0.3),
                                  dirs=dirs)
        origs = np.tile(np.array(model.orig, np.float64), (3000, 1))
    else:
        o = rng.uniform(-0.3, 0.3, (3000, 3)).astype(np.float32)
        model = sensors.OnDnModel(width=60, height=50, range=sensors.Interval(0.3, 130.0), origs=o, dirs=dirs)
        origs = o.astype(np.float64)
    Tsb = np.array([0, 0, np.sin(0.1), np.cos(0.1), 0.1, 0.05, 0.4, 0], np.float32)
    m = rm.Map(sc.vertices, sc.faces)
    sim = rm.make_simulator(model, m)
    sim.setTsb(Tsb)
    assert sim.sensor.visit_order() is not None
    obs = sim.simulate(torch.from_numpy(true).cuda(), attrs=("ranges",)).ranges
    g, loss, rs, fs = rg.range_pose_grad(sim, torch.from_numpy(est).cuda(), obs, DELTA, want_sim=True)
    torch.cuda.synchronize()
    g, loss = g.cpu().numpy(), loss.cpu().numpy()
    rs, fs, ob = rs.cpu().numpy(), fs.cpu().numpy().view(np.uint32), obs.cpu().numpy()
    rmin, rmax = model.range.min, model.range.max
    valid = (fs != 0xFFFFFFFF) & (rs >= rmin) & (ob >= rmin) & (ob <= rmax)
    gid = np.nonzero(valid)[0]
    assert gid.size > 0.3 * fs.size
    rset = og.RayFaceSet(sc.vertices, sc.faces, Tsb, est, dirs[gid % 3000], origs[gid % 3000], gid // 3000,
                         fs[gid], ob[gid])
    an, an_loss = rset.analytic(est.shape[0], DELTA)
    assert np.abs(g - an).max() / np.abs(an).max() < 1e-3
    assert np.abs(loss - an_loss).max() / np.abs(an_loss).max() < 1e-3
    assert m.status() == 0
