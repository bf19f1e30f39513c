"""The 3x3 SVD (rmg_svd3), the Umeyama step and its backward on the inputs that ICP meets on terrain
and in rooms: random matrices as in rmagine's own SVD tests (tests/core/math_svd.cpp:161-237,
tests/cuda/math_svd.cpp:38-109, which check U W V^T against A), and rank-deficient (coplanar,
collinear, one correspondence), repeated and reflected singular values, checked against numpy's
binary64 SVD and the binary64 Umeyama oracle (oracle/stats.py).  Backward gradients are checked
against binary64 central differences where the rotation is differentiable, and for boundedness
where it is not."""
import zlib

import numpy as np
import pytest

from oracle import stats as ost

F32 = np.float32
gpu = pytest.mark.gpu


@pytest.fixture(scope="module")
def rs(built):
    import torch

    from rmagine_gb300 import statistics

    torch.cuda.set_device(0)
    return statistics


def rot(q):
    return ost.quat_to_rot(np.asarray(q, np.float64))


def random_rotations(rng, n):
    q = rng.standard_normal((n, 4))
    return rot(q / np.linalg.norm(q, axis=1, keepdims=True))


def from_singular_values(rng, sv, n):
    """n matrices Ru diag(sv) Rv^T with random rotations Ru, Rv (sv may carry a negative last value:
    a reflection)."""
    Ru, Rv = random_rotations(rng, n), random_rotations(rng, n)
    return np.einsum("bij,j,bkj->bik", Ru, np.asarray(sv, np.float64), Rv)


def run_svd(rs, A, rotations=False):
    import torch

    U, w, V = rs.svd(torch.from_numpy(np.ascontiguousarray(A, F32)).cuda(), rotations=rotations)
    torch.cuda.synchronize()
    return U.cpu().numpy().astype(np.float64), w.cpu().numpy().astype(np.float64), V.cpu().numpy().astype(np.float64)


def check_svd(rs, A, name):
    A = np.asarray(A, F32).astype(np.float64)  # the matrices the GPU sees
    scale = np.maximum(np.abs(A).max(axis=(1, 2)), 1e-30)
    ref = np.linalg.svd(A, compute_uv=False)
    for rotations in (False, True):
        U, w, V = run_svd(rs, A, rotations)
        rec = np.einsum("bij,bj,bkj->bik", U, w, V)
        assert (np.abs(rec - A).max(axis=(1, 2)) / scale).max() < 2e-6, (name, rotations)
        for M in (U, V):
            assert np.abs(np.einsum("bji,bjk->bik", M, M) - np.eye(3)).max() < 2e-6, (name, rotations)
        # singular values are unique: compare with numpy's binary64 SVD (sorted, non-negative)
        assert (np.abs(np.abs(w) - ref).max(axis=1) / np.maximum(ref[:, 0], 1e-30)).max() < 2e-6, (name, rotations)
        tol = 2e-6 * np.maximum(ref[:, :1], 1e-30)
        assert np.all(w[:, 0:1] >= w[:, 1:2] - tol) and np.all(w[:, 1:2] >= np.abs(w[:, 2:3]) - tol), name
        if rotations:
            assert np.abs(np.linalg.det(U) - 1).max() < 1e-5 and np.abs(np.linalg.det(V) - 1).max() < 1e-5, name
            detA = np.linalg.det(A)
            sure = np.abs(detA) > 1e-3 * scale ** 3  # sign of a (near-)singular matrix is noise
            assert np.all(np.sign(w[sure, 2]) == np.sign(detA[sure])), name
        else:
            assert np.all(w >= 0), name


@gpu
def test_svd_random_matrices_reconstruct(rs):
    # Eigen::Matrix3f::Random: uniform in [-1, 1], as in rmagine's SVD accuracy and GPU tests
    rng = np.random.default_rng(0)
    check_svd(rs, rng.uniform(-1, 1, (100_000, 3, 3)), "uniform[-1,1]")
    check_svd(rs, rng.standard_normal((20_000, 3, 3)) * 1e3, "gaussian * 1e3")


@gpu
@pytest.mark.parametrize("name,sv", [
    ("rank 2 (coplanar)", (3.0, 1.0, 0.0)),
    ("rank 2, thin", (1.0, 1e-4, 0.0)),
    ("rank 1 (collinear)", (2.0, 0.0, 0.0)),
    ("zero", (0.0, 0.0, 0.0)),
    ("three equal", (1.5, 1.5, 1.5)),
    ("two equal, large", (2.0, 2.0, 0.5)),
    ("two equal, small", (2.0, 0.5, 0.5)),
    ("reflection", (3.0, 2.0, -1.0)),
    ("reflection, two equal", (3.0, 1.0, -1.0)),
    ("condition 1e6", (1.0, 1e-3, 1e-6)),
    ("large entries", (1e6, 3e5, 1e5)),
    ("small entries", (1e-6, 3e-7, 1e-7)),
])
def test_svd_structured_matrices(rs, name, sv):
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    check_svd(rs, from_singular_values(rng, sv, 4096), name)


@gpu
def test_svd_signed_permutations(rs):
    mats = [np.eye(3)[list(p)] * d for p in [(0, 1, 2), (1, 0, 2), (2, 1, 0), (1, 2, 0), (2, 0, 1)] for d in (1, -1, 3)]
    mats += [np.diag([1.0, -2.0, 3.0]), np.diag([0.0, 5.0, 0.0]), np.diag([-1.0, -1.0, -1.0])]
    check_svd(rs, np.array(mats), "signed permutations and diagonals")


# ---- Umeyama on degenerate correspondence sets ------------------------------------------------
def rigid(rng, pts, R, t):
    return np.einsum("ij,bnj->bni", R, pts) + t


def umeyama_gpu(rs, src, tgt, mask=None):
    import torch

    s, T = rs.statistics(src.astype(F32), tgt.astype(F32), dataset_mask=mask)
    torch.cuda.synchronize()
    T = T.cpu().numpy().astype(np.float64)
    return ost.quat_to_rot(T[:, :4]), T[:, 4:7], T, s


@gpu
def test_umeyama_recovers_the_pose_on_coplanar_and_isotropic_sets(rs):
    rng = np.random.default_rng(3)
    R = random_rotations(rng, 1)[0]
    t = rng.uniform(-5, 5, 3)
    N = 64
    sets = []
    plane = np.zeros((N, 3))
    plane[:, :2] = rng.uniform(-10, 10, (N, 2))
    sets.append(plane)  # coplanar (a floor): rank-2 covariance
    tri = np.zeros((N, 3))
    tri[:3] = [[1, 0, 0], [0, 2, 0], [-1, -1, 0.5]]
    sets.append(tri)  # three correspondences (the rest masked out)
    iso = np.zeros((N, 3))
    iso[:6] = np.concatenate([np.eye(3), -np.eye(3)]) * 2.0
    sets.append(iso)  # three equal singular values
    strip = np.zeros((N, 3))
    strip[:, 0] = rng.uniform(-20, 20, N)
    strip[:, 1] = rng.uniform(-0.05, 0.05, N)
    sets.append(strip)  # coplanar and thin (a corridor wall seen edge-on)
    src = np.stack(sets)
    tgt = rigid(rng, src, R, t)
    mask = np.ones((len(sets), N), np.uint8)
    mask[1, 3:] = 0
    mask[2, 6:] = 0
    Rg, tg, _, _ = umeyama_gpu(rs, src, tgt, mask)
    ang = ost.rotation_angle(np.broadcast_to(R, Rg.shape), Rg)
    # float32 points: the strip's thin axis is resolved to about 6e-8 * 20 / 0.05 rad
    assert ang[:3].max() < 2e-6, ang
    assert ang[3] < 1e-4, ang
    assert np.abs(np.linalg.det(Rg) - 1).max() < 1e-5
    assert np.abs(tg[:3] - t).max() < 2e-5


@gpu
def test_umeyama_on_collinear_single_and_empty_sets(rs):
    rng = np.random.default_rng(4)
    R = random_rotations(rng, 1)[0]
    t = rng.uniform(-5, 5, 3)
    N = 32
    line_dir = np.array([0.3, -0.5, 0.8]) / np.linalg.norm([0.3, -0.5, 0.8])
    src = np.zeros((4, N, 3))
    src[0] = rng.uniform(-10, 10, (N, 1)) * line_dir + [1, 2, 3]  # collinear
    src[1, :2] = [[0, 0, 0], [2, 1, -1]]                             # two correspondences
    src[2, 0] = [4, -2, 1]                                           # one correspondence
    tgt = rigid(rng, src, R, t)
    mask = np.ones((4, N), np.uint8)
    mask[1, 2:] = 0
    mask[2, 1:] = 0
    mask[3, :] = 0                                                   # none: identity
    Rg, tg, T, s = umeyama_gpu(rs, src, tgt, mask)
    assert np.all(np.isfinite(T))
    assert np.abs(np.linalg.det(Rg) - 1).max() < 1e-5
    # a line fixes the rotation only up to a spin about itself: R must map the line onto the line
    for b, d in ((0, line_dir), (1, np.array([2.0, 1.0, -1.0]) / np.sqrt(6.0))):
        md = R @ d
        got = Rg[b] @ d
        assert np.arccos(np.clip(abs(got @ md), -1, 1)) < 1e-5, b
        m_mean = tgt[b][mask[b] > 0].mean(axis=0)
        d_mean = src[b][mask[b] > 0].mean(axis=0)
        assert np.abs(tg[b] - (m_mean - Rg[b] @ d_mean)).max() < 1e-4, b
    # one correspondence: zero covariance; the identity rotation and t = m - d fit it exactly
    assert np.abs(Rg[2] - np.eye(3)).max() < 1e-6
    assert np.abs(tg[2] - (tgt[2, 0] - src[2, 0])).max() < 1e-5
    assert np.array_equal(T[3], np.array([0, 0, 0, 1, 0, 0, 0, 0], np.float64))


@gpu
def test_umeyama_reflected_sets_match_the_oracle(rs):
    # the model is a mirror image of the dataset: the best proper rotation (reflection fix of
    # optimization.cpp:25-29) is found, as by the binary64 oracle
    rng = np.random.default_rng(5)
    N = 256
    X = rng.standard_normal((6, N, 3)) * [4.0, 2.0, 1.0]
    M = np.diag([1.0, 1.0, -1.0])
    R = random_rotations(rng, 6)
    src = X
    tgt = np.einsum("bij,jk,bnk->bni", R, M, X) + rng.uniform(-3, 3, (6, 1, 3))
    Rg, tg, _, _ = umeyama_gpu(rs, src, tgt)
    want = ost.stats(*ost.correspondences(src.astype(F32), tgt.astype(F32)))
    Ro, to, _ = ost.umeyama(want)
    assert ost.rotation_angle(Ro, Rg).max() < 2e-6
    assert np.abs(tg - to).max() < 2e-5


# ---- backward near and at the rotation's singular configurations -----------------------------
def exact_cov_cloud(rng, N, var, Rv):
    """N points whose sample covariance is exactly Rv diag(var) Rv^T (before rounding to binary32)."""
    X = rng.standard_normal((N, 3))
    X -= X.mean(axis=0)
    L = np.linalg.cholesky(X.T @ X / N)
    X = X @ np.linalg.inv(L).T * np.sqrt(var)
    return X @ Rv.T


def backward(rs, src, tgt, gR, gt):
    import torch

    s, _ = rs.statistics(src.astype(F32), tgt.astype(F32))
    gd, gm = rs.umeyama_backward(src.astype(F32), tgt.astype(F32), s, grad_R=gR.astype(F32), grad_t=gt.astype(F32))
    torch.cuda.synchronize()
    return gd.cpu().numpy().astype(np.float64), gm.cpu().numpy().astype(np.float64)


@gpu
@pytest.mark.parametrize("case", ["coplanar", "coplanar thin", "reflection gap 1e-1", "reflection gap 1e-2",
                                  "reflection gap 3e-3"])
def test_umeyama_backward_near_singular_matches_finite_differences(rs, case):
    rng = np.random.default_rng(zlib.crc32(case.encode()))
    N = 24
    Rv = random_rotations(rng, 1)[0]
    R = random_rotations(rng, 1)[0]
    t = rng.uniform(-2, 2, 3)
    if case.startswith("coplanar"):
        var = [4.0, 1.0 if case == "coplanar" else 0.05, 0.0]
        X = exact_cov_cloud(rng, N, np.maximum(var, 1e-30), Rv)
        tgt = X @ R.T + t + rng.normal(0, 0.01, (N, 3))
    else:
        gap = float(case.split()[-1])
        X = exact_cov_cloud(rng, N, [4.0, 1.0, 1.0 - gap], Rv)
        # mirror in the frame of the cloud: the optimal proper rotation has s2 + s3 = gap * s2
        tgt = X @ (R @ Rv @ np.diag([1.0, 1.0, -1.0]) @ Rv.T).T + t
    src, tgt = X[None].astype(F32), tgt[None].astype(F32)
    gR = rng.standard_normal((1, 3, 3))
    gt = rng.standard_normal((1, 3))
    gd, gm = backward(rs, src, tgt, gR, gt)
    fd, fm = ost.loss_fd_gradients(src, tgt, gR, gt, h=1e-5)
    for g, f in ((gd, fd), (gm, fm)):
        err = np.abs(g - f).max() / np.abs(f).max()
        assert err < 1e-3, (case, err)


@gpu
def test_umeyama_backward_is_bounded_where_the_rotation_is_not_unique(rs):
    # collinear points (s2 = s3 = 0) and a mirrored cloud with two equal spreads (s2 = -s3): the
    # rotation about one axis is not determined, that component gets no gradient, and the rest stays
    # finite and of the order of the upstream gradient over the cloud's extent
    rng = np.random.default_rng(7)
    N = 24
    R = random_rotations(rng, 1)[0]
    line = np.outer(rng.uniform(-3, 3, N), [0.6, 0.0, 0.8]) + [1.0, -1.0, 0.5]
    Rv = random_rotations(rng, 1)[0]
    mirror = exact_cov_cloud(rng, N, [4.0, 1.0, 1.0], Rv)
    cases = [(line, line @ R.T), (mirror, mirror @ (R @ Rv @ np.diag([1.0, 1.0, -1.0]) @ Rv.T).T)]
    for src, tgt in cases:
        gR = rng.standard_normal((1, 3, 3))
        gt = rng.standard_normal((1, 3))
        gd, gm = backward(rs, src[None], tgt[None], gR, gt)
        for g in (gd, gm):
            assert np.all(np.isfinite(g))
            assert np.abs(g).max() < 1e2, np.abs(g).max()
