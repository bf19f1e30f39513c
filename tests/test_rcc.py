"""rmagine's pose-correction integration test (tests/embree/correction_rcc.cpp:60-180): simulate a
scan at the true pose, start 0.1 m / 0.1 rad off, and alternate simulate -> statistics_p2l ->
Umeyama (10 x 5 iterations); the estimate must converge to |dz|, |dyaw| < 1e-3.  Run with the
oracle (CPU) and with the GPU library."""
import math

import numpy as np
import pytest

from rmagine_gb300 import scenes, sensors, transforms

DEG = 0.017453292519943295


def rcc_model():
    """correction_rcc.cpp:68-82: 32 x 360 spherical, phi from -64 deg in 4 deg steps."""
    f = sensors.f32
    F = float(np.float32(DEG))
    return sensors.SphericalModel(phi=sensors.DiscreteInterval(f(-64.0 * F), f(4.0 * F), 32),
                                  theta=sensors.DiscreteInterval(f(-math.pi), f(1.0 * F), 360),
                                  range=sensors.Interval(0.5, 130.0))


def start_pose():
    T = transforms.identity()
    T[:4] = scenes.euler_to_quat([0.0], [0.0], [0.1])[0]
    T[6] = 0.1
    return T


def converged(T_est):
    Tdiff = transforms.compose(transforms.inverse(T_est), transforms.identity())
    return abs(float(Tdiff[6])) < 1e-3 and abs(float(transforms.yaw(Tdiff[:4]))) < 1e-3


def test_rcc_correction_oracle():
    import oracle
    from oracle import stats as ost

    v, f = scenes.gen_cube()
    sc = oracle.Scene(v, f)
    model = rcc_model()
    ident = transforms.identity()
    data = sc.simulate(model, ident, ident[None], attrs=("hits", "points"))
    T_est = start_pose()
    for _ in range(10):
        mod = sc.simulate(model, ident, T_est[None], attrs=("hits", "points", "normals"))
        Tpre = transforms.identity()
        for _ in range(5):
            D, M, ok = ost.correspondences(data["points"][None], mod["points"][None], Tpre,
                                           dmask=data["hits"][None], mmask=mod["hits"][None], max_dist=100.0,
                                           normals=mod["normals"][None])
            R, t, q = ost.umeyama(ost.stats(D, M, ok))
            Tn = transforms.identity()
            Tn[:4] = q[0]
            Tn[4:7] = t[0]
            Tpre = transforms.compose(Tpre, Tn)
        T_est = transforms.compose(T_est, Tpre)
    assert converged(T_est), T_est


@pytest.mark.gpu
def test_rcc_correction_gpu(built):
    import torch

    import rmagine_gb300 as rm
    from rmagine_gb300 import statistics as rs

    torch.cuda.set_device(0)
    v, f = scenes.gen_cube()
    m = rm.Map(v, f)
    sim = rm.SphereSimulator(m)
    sim.setModel(rcc_model())
    data = sim.simulate(torch.from_numpy(transforms.identity(1)).cuda(), attrs=("hits", "points"))
    T_est = start_pose()
    P = rs.UmeyamaReductionConstraints(max_dist=100.0)
    for _ in range(10):
        mod = sim.simulate(torch.from_numpy(T_est[None].copy()).cuda(), attrs=("hits", "points", "normals"))
        Tpre = transforms.identity()
        for _ in range(5):
            _, T = rs.statistics_p2l(data.points[None], mod.points[None], mod.normals[None], pre=Tpre, params=P,
                                     dataset_mask=data.hits[None], model_mask=mod.hits[None])
            Tpre = transforms.compose(Tpre, T[0].cpu().numpy())
        T_est = transforms.compose(T_est, Tpre)
    assert converged(T_est), T_est
