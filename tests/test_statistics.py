"""CrossStatistics -> Umeyama (forward and backward): oracle pins on the CPU, GPU parity against
the binary64 oracle."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import stats as ost

GOLD = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())
F32 = np.float32


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def paper_batch():
    g = GOLD["cross_stats_paper"]
    d = np.array([p["dataset_mean"] for p in g["inputs"]], F32)[None]
    m = np.array([p["model_mean"] for p in g["inputs"]], F32)[None]
    return d, m, g["expect"]


def filter_case(n):
    """tests/core/math_statistics.cpp:495-509 data."""
    i = np.arange(n)
    p = (i.astype(np.float64) / float(n)).astype(F32)
    d = np.stack([-p, p * F32(10), p], 1).astype(F32)
    m = np.stack([p, p, -p], 1).astype(F32)
    return d[None], m[None], (i % 2).astype(np.uint8)[None], (i % 4).astype(np.uint32)[None]


def icp_batches(B, N, seed, outliers=0.05):
    """Source points uniform in a 50 m cube; targets = R src + t + N(0, 0.01) with a fraction of
    outliers displaced by U(-5, 5) per axis; per-batch random R (uniform quaternion), t ~ U(-5, 5)."""
    rng = np.random.default_rng(seed)
    src = rng.uniform(-25, 25, (B, N, 3))
    q = rng.standard_normal((B, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    R = ost.quat_to_rot(q)
    t = rng.uniform(-5, 5, (B, 3))
    tgt = np.einsum("bij,bnj->bni", R, src) + t[:, None, :] + rng.normal(0, 0.01, (B, N, 3))
    out = rng.random((B, N)) < outliers
    tgt[out] += rng.uniform(-5, 5, (int(out.sum()), 3))
    return src.astype(F32), tgt.astype(F32), R, t


# ---- CPU: pin the oracle -------------------------------------------------------------
def test_oracle_paper_example():
    d, m, e = paper_batch()
    st = ost.stats(*ost.correspondences(d, m))
    assert abs(st["dataset_mean"][0, 0] - e["dataset_mean"][0]) < 1e-4
    assert abs(st["model_mean"][0, 0] - e["model_mean"][0]) < 1e-4
    assert abs(st["covariance"][0, 0, 0] - e["cov00"]) < 1e-4
    assert st["n"][0] == e["n_meas"]


def test_oracle_filter_counts():
    g = GOLD["p2p_filter_counts"]
    d, m, mask, ids = filter_case(g["n_points"])
    md = g["max_dist"]
    assert ost.stats(*ost.correspondences(d, m, max_dist=md))["n"][0] == g["cases"][0]["expect"]
    assert ost.stats(*ost.correspondences(d, m, dmask=mask, max_dist=md))["n"][0] == g["cases"][1]["expect"]
    assert ost.stats(*ost.correspondences(d, m, dmask=mask, dids=ids, dataset_id=2, max_dist=md))["n"][0] == \
        g["cases"][2]["expect"]


def test_oracle_umeyama_recovers_rigid_motion():
    src, tgt, R, t = icp_batches(8, 2000, seed=1, outliers=0.0)
    Ro, to, q = ost.umeyama(ost.stats(*ost.correspondences(src, tgt)))
    assert ost.rotation_angle(Ro, R).max() < 1e-4
    assert np.abs(to - t).max() < 1e-3
    assert np.allclose(ost.quat_to_rot(q), Ro, atol=1e-12)


def test_oracle_merge_matches_reference_fold(ref_lib):
    """rmagine's incremental CrossStatistics merge (binary32), compiled from its headers, against
    the oracle's binary64 two-pass statistics, with the reference test's own equality tolerances
    (tests/core/math_statistics.cpp:72-104)."""
    src, tgt, _, _ = icp_batches(1, 1000, seed=2)
    out = np.zeros(15, F32)
    n = np.zeros(1, np.uint32)
    ref_lib.ref_cross_stats_fold(_p(np.ascontiguousarray(src[0])), _p(np.ascontiguousarray(tgt[0])), C.c_uint32(1000),
                                 _p(out), _p(n))
    st = ost.stats(*ost.correspondences(src, tgt))
    assert n[0] == st["n"][0]
    assert np.linalg.norm(out[0:3] - st["dataset_mean"][0]) < 1e-4
    assert np.linalg.norm(out[3:6] - st["model_mean"][0]) < 1e-3
    cov_ref = out[6:15].reshape(3, 3).T  # column-major
    assert np.abs(cov_ref - st["covariance"][0]).mean() / np.abs(st["covariance"][0]).max() < 1e-4


def test_oracle_rot_to_quat_matches_reference(ref_lib):
    rng = np.random.default_rng(3)
    q = rng.standard_normal((200, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    Rm = ost.quat_to_rot(q).astype(F32)
    ref = np.zeros((200, 4), F32)
    ref_lib.ref_matrix_to_quat(_p(np.ascontiguousarray(Rm.reshape(200, 9))), _p(ref), C.c_uint32(200))
    mine = ost.rot_to_quat(Rm.astype(np.float64))
    ref /= np.linalg.norm(ref, axis=1, keepdims=True)
    assert np.abs(mine - ref).max() < 1e-5  # same branch -> same sign


# ---- GPU -----------------------------------------------------------------------------------
gpu = pytest.mark.gpu


@pytest.fixture(scope="module")
def rs(built):
    import torch

    from rmagine_gb300 import statistics as rs_

    torch.cuda.set_device(0)
    return rs_


def gpu_stats(rs, *a, **k):
    import torch

    s, T = rs.statistics(*a, **k)
    torch.cuda.synchronize()
    return rs.decode_stats(s), (None if T is None else T.cpu().numpy())


def check_stats(got, want, cov_rel=2e-6, mean_abs=2e-5):
    assert np.array_equal(got["n"], want["n"])
    assert np.abs(got["dataset_mean"] - want["dataset_mean"]).max() <= mean_abs * (1 + np.abs(want["dataset_mean"]).max())
    assert np.abs(got["model_mean"] - want["model_mean"]).max() <= mean_abs * (1 + np.abs(want["model_mean"]).max())
    scale = np.abs(want["covariance"]).max(axis=(1, 2), keepdims=True) + 1e-30
    assert (np.abs(got["covariance"] - want["covariance"]) / scale).max() <= cov_rel


@gpu
def test_gpu_paper_example(rs):
    d, m, e = paper_batch()
    got, T = gpu_stats(rs, d, m)
    assert abs(got["dataset_mean"][0, 0] - 5.0) < 1e-6 and abs(got["model_mean"][0, 0] - 4.0) < 1e-6
    assert abs(got["covariance"][0, 0, 0] - 4.0) < 1e-6 and got["n"][0] == 4


@gpu
def test_gpu_filter_counts_single_large_batch(rs):
    """1M correspondences in one batch: exercises the multi-CTA split of a batch."""
    g = GOLD["p2p_filter_counts"]
    d, m, mask, ids = filter_case(g["n_points"])
    P = rs.UmeyamaReductionConstraints(max_dist=g["max_dist"])
    assert gpu_stats(rs, d, m, params=P)[0]["n"][0] == g["cases"][0]["expect"]
    assert gpu_stats(rs, d, m, params=P, dataset_mask=mask)[0]["n"][0] == g["cases"][1]["expect"]
    P2 = rs.UmeyamaReductionConstraints(max_dist=g["max_dist"], dataset_id=2)
    got, T = gpu_stats(rs, d, m, params=P2, dataset_mask=mask, dataset_ids=ids)
    assert got["n"][0] == 0
    assert np.array_equal(T[0], np.array([0, 0, 0, 1, 0, 0, 0, 0], F32))  # n == 0 -> identity
    want = ost.stats(*ost.correspondences(d, m, max_dist=g["max_dist"]))
    check_stats(gpu_stats(rs, d, m, params=P)[0], want)


@gpu
@pytest.mark.parametrize("N", [4096, 1001])  # vector path and scalar path
def test_gpu_stats_and_umeyama_match_fp64_oracle(rs, N):
    B = 64
    src, tgt, R, t = icp_batches(B, N, seed=4)
    # max_dist = 1 m on clouds pre-aligned by the true pose (the ICP case): the filter drops the
    # outliers and keeps the inliers
    pre = np.zeros((B, 8), F32)
    pre[:, :4] = ost.rot_to_quat(R)
    pre[:, 4:7] = t
    for md, pr in ((np.inf, None), (1.0, pre)):
        P = rs.UmeyamaReductionConstraints(max_dist=md)
        got, T = gpu_stats(rs, src, tgt, pre=pr, params=P)
        want = ost.stats(*ost.correspondences(src, tgt, pr, max_dist=md))
        assert want["n"].min() > 0.9 * N
        check_stats(got, want)
        Ro, to, qo = ost.umeyama(want)
        Rg = ost.quat_to_rot(T[:, :4].astype(np.float64))
        assert ost.rotation_angle(Rg, Ro).max() < (2e-6 if pr is None else 2e-5)
        assert np.abs(T[:, 4:7] - to).max() < 2e-5 * (1 + np.abs(to).max())
        # the quaternion sign follows the reference's branch order
        assert np.abs(T[:, :4] - qo).max() < 1e-5


@gpu
def test_gpu_pre_transform_masks_ids_and_p2l(rs):
    B, N = 16, 2048
    src, tgt, R, t = icp_batches(B, N, seed=5)
    rng = np.random.default_rng(6)
    pre = np.zeros((B, 8), F32)
    pre[:, :4] = ost.rot_to_quat(ost.quat_to_rot(rng.standard_normal((B, 4)) / 4 + [0, 0, 0, 1]))
    pre[:, 4:7] = rng.uniform(-1, 1, (B, 3))
    dmask = (rng.random((B, N)) < 0.8).astype(np.uint8)
    mmask = (rng.random((B, N)) < 0.9).astype(np.uint8)
    mids = rng.integers(0, 3, (B, N)).astype(np.uint32)
    P = rs.UmeyamaReductionConstraints(max_dist=20.0, model_id=1)
    got, T = gpu_stats(rs, src, tgt, pre=pre, params=P, dataset_mask=dmask, model_mask=mmask, model_ids=mids)
    want = ost.stats(*ost.correspondences(src, tgt, pre, dmask=dmask, mmask=mmask, mids=mids, model_id=1,
                                          max_dist=20.0))
    check_stats(got, want)
    # one pre-transform for all batches (stride 0)
    got, _ = gpu_stats(rs, src, tgt, pre=pre[0], params=P)
    want = ost.stats(*ost.correspondences(src, tgt, pre[0], max_dist=20.0))
    check_stats(got, want)
    # point-to-plane
    nrm = rng.standard_normal((B, N, 3))
    nrm = (nrm / np.linalg.norm(nrm, axis=2, keepdims=True)).astype(F32)
    P = rs.UmeyamaReductionConstraints(max_dist=2.0)
    got, T = gpu_stats(rs, src, tgt, pre=pre, params=P, model_normals=nrm)
    want = ost.stats(*ost.correspondences(src, tgt, pre, max_dist=2.0, normals=nrm))
    check_stats(got, want, cov_rel=1e-5)


@gpu
def test_gpu_umeyama_from_stats_matches_fused(rs):
    import torch

    src, tgt, _, _ = icp_batches(32, 1024, seed=7)
    s, T = rs.statistics(src, tgt)
    T2 = rs.umeyama_transform(s)
    torch.cuda.synchronize()
    Ra = ost.quat_to_rot(T.cpu().numpy()[:, :4].astype(np.float64))
    Rb = ost.quat_to_rot(T2.cpu().numpy()[:, :4].astype(np.float64))
    assert ost.rotation_angle(Ra, Rb).max() < 1e-5


@gpu
def test_gpu_umeyama_backward_matches_finite_differences(rs):
    import torch

    B, N = 4, 24
    src, tgt, _, _ = icp_batches(B, N, seed=8, outliers=0.0)
    rng = np.random.default_rng(9)
    pre = np.zeros((B, 8), F32)
    pre[:, :4] = ost.rot_to_quat(ost.quat_to_rot(rng.standard_normal((B, 4)) / 5 + [0, 0, 0, 1]))
    pre[:, 4:7] = rng.uniform(-0.5, 0.5, (B, 3))
    gR = rng.standard_normal((B, 3, 3))
    gt = rng.standard_normal((B, 3))
    mask = np.ones((B, N), np.uint8)
    mask[:, 3] = 0  # a filtered correspondence gets zero gradient
    s, _ = rs.statistics(src, tgt, pre=pre, dataset_mask=mask)
    gd, gm = rs.umeyama_backward(src, tgt, s, grad_R=gR.astype(F32), grad_t=gt.astype(F32), pre=pre,
                                 dataset_mask=mask)
    torch.cuda.synchronize()
    gd, gm = gd.cpu().numpy(), gm.cpu().numpy()
    fd, fm = ost.loss_fd_gradients(src, tgt, gR, gt, pre=pre, dmask=mask)
    assert np.all(gd[:, 3] == 0) and np.all(gm[:, 3] == 0)
    for g, f in ((gd, fd), (gm, fm)):
        err = np.abs(g - f).max() / np.abs(f).max()
        assert err < 1e-3, err
