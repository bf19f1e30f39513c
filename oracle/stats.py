"""ORACLE -- test infrastructure only.  Binary64 restatement of rmagine's
correspondence statistics and Umeyama step, plus finite-difference gradients.

* statistics_p2p / statistics_p2l: src/rmagine_core/src/math/statistics.cpp:19-126 (filters as
  in the GPU kernels src/rmagine_cuda/src/math/statistics.cu:58-140 (squared p2p distance) and
  :190-276).  The pre-transform and the filter run in binary32 in the same operation order as
  the reference (Transform * Vector = q (v,0) q^-1 + t); accumulation is exact-ish binary64
  (two-pass mean / covariance).
* umeyama: src/rmagine_core/src/math/optimization.cpp:12-49 with numpy's binary64 SVD:
  R = U diag(1, 1, sign det(U V^T)) V^T, t = m - R d; n == 0 -> identity.
* CrossStatistics: covariance = (1/n) sum (m - m_mean)(d - d_mean)^T (CrossStatistics.tcc:7-58).
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def _qmul(a, b):
    """Quaternion.tcc:35-42 in binary32, term order kept."""
    ax, ay, az, aw = (a[..., k] for k in range(4))
    bx, by, bz, bw = (b[..., k] for k in range(4))
    x = ((aw * bx + ax * bw) + ay * bz) - az * by
    y = ((aw * by - ax * bz) + ay * bw) + az * bx
    z = ((aw * bz + ax * by) - ay * bx) + az * bw
    w = ((aw * bw - ax * bx) - ay * by) - az * bz
    return np.stack([x, y, z, w], axis=-1).astype(F32)


def transform_points_f32(T, p):
    """rmagine Transform * Vector3 in binary32: rotate by q (v,0) q^-1, then add t.
    T: [..., 8] transform records, p: [..., 3]."""
    T = np.asarray(T, F32)
    p = np.asarray(p, F32)
    q = np.broadcast_to(T[..., :4], p.shape[:-1] + (4,)).astype(F32)
    P = np.concatenate([p, np.zeros(p.shape[:-1] + (1,), F32)], axis=-1)
    qi = q * np.array([-1, -1, -1, 1], F32)
    r = _qmul(_qmul(q, P), qi)
    t = np.broadcast_to(T[..., 4:7], p.shape).astype(F32)
    return (r[..., :3] + t).astype(F32)


def correspondences(dataset, model, pre=None, dmask=None, mmask=None, dids=None, mids=None, dataset_id=0,
                    model_id=0, max_dist=np.inf, normals=None):
    """Per batch: binary32 pre-transformed dataset points D, model correspondences M, validity.
    dataset/model: [B, N, 3] float32; pre: [8] or [B, 8] or None."""
    dataset = np.asarray(dataset, F32)
    model = np.asarray(model, F32)
    Bn, N, _ = dataset.shape
    if pre is None:
        D = dataset.copy()
    else:
        pre = np.asarray(pre, F32).reshape(-1, 8)
        T = np.broadcast_to(pre[:, None, :] if pre.shape[0] == Bn else pre[0][None, None, :], (Bn, N, 8))
        D = transform_points_f32(T, dataset)
    ok = np.ones((Bn, N), bool)
    if dmask is not None:
        ok &= np.asarray(dmask).reshape(Bn, N) > 0
    if mmask is not None:
        ok &= np.asarray(mmask).reshape(Bn, N) > 0
    if dids is not None:
        ok &= np.asarray(dids).reshape(Bn, N) == dataset_id
    if mids is not None:
        ok &= np.asarray(mids).reshape(Bn, N) == model_id
    md = F32(max_dist)
    if normals is None:
        M = model
        diff = (M - D).astype(F32)
        d2 = (diff[..., 0] * diff[..., 0] + diff[..., 1] * diff[..., 1]) + diff[..., 2] * diff[..., 2]
        ok &= d2 < F32(md * md)
    else:
        Nn = np.asarray(normals, F32)
        diff = (model - D).astype(F32)
        sd = (diff[..., 0] * Nn[..., 0] + diff[..., 1] * Nn[..., 1]) + diff[..., 2] * Nn[..., 2]
        ok &= np.abs(sd) < md
        M = (D + Nn * sd[..., None]).astype(F32)
    return D, M, ok


def stats(D, M, ok):
    """Binary64 CrossStatistics per batch: dict of dataset_mean [B,3], model_mean [B,3],
    covariance [B,3,3] (row i = model axis, col j = dataset axis), n [B]."""
    # masked-out entries may hold NaN (miss rays carry NaN points): select, do not multiply by 0
    D = np.where(ok[..., None], D.astype(np.float64), 0.0)
    M = np.where(ok[..., None], M.astype(np.float64), 0.0)
    w = ok.astype(np.float64)
    n = w.sum(axis=1)
    nn = np.maximum(n, 1.0)[:, None]
    dm = (D * w[..., None]).sum(axis=1) / nn
    mm = (M * w[..., None]).sum(axis=1) / nn
    dc = (D - dm[:, None, :]) * w[..., None]
    mc = (M - mm[:, None, :]) * w[..., None]
    C = np.einsum("bni,bnj->bij", mc, dc) / nn[..., None]
    zero = n == 0
    dm[zero] = 0
    mm[zero] = 0
    C[zero] = 0
    return {"dataset_mean": dm, "model_mean": mm, "covariance": C, "n": n.astype(np.int64)}


def rot_to_quat(R):
    """Rotation matrix -> (x, y, z, w), branch order of MatrixOps.tcc:1492-1529, normalised."""
    R = np.asarray(R, np.float64)
    q = np.zeros(R.shape[:-2] + (4,))
    for idx in np.ndindex(R.shape[:-2]):
        m = R[idx]
        tr = m[0, 0] + m[1, 1] + m[2, 2]
        if tr > 0:
            S = np.sqrt(tr + 1.0) * 2
            v = [(m[2, 1] - m[1, 2]) / S, (m[0, 2] - m[2, 0]) / S, (m[1, 0] - m[0, 1]) / S, 0.25 * S]
        elif m[0, 0] > m[1, 1] and m[0, 0] > m[2, 2]:
            S = np.sqrt(1.0 + m[0, 0] - m[1, 1] - m[2, 2]) * 2
            v = [0.25 * S, (m[0, 1] + m[1, 0]) / S, (m[0, 2] + m[2, 0]) / S, (m[2, 1] - m[1, 2]) / S]
        elif m[1, 1] > m[2, 2]:
            S = np.sqrt(1.0 + m[1, 1] - m[0, 0] - m[2, 2]) * 2
            v = [(m[0, 1] + m[1, 0]) / S, 0.25 * S, (m[1, 2] + m[2, 1]) / S, (m[0, 2] - m[2, 0]) / S]
        else:
            S = np.sqrt(1.0 + m[2, 2] - m[0, 0] - m[1, 1]) * 2
            v = [(m[0, 2] + m[2, 0]) / S, (m[1, 2] + m[2, 1]) / S, 0.25 * S, (m[1, 0] - m[0, 1]) / S]
        v = np.array(v)
        q[idx] = v / np.linalg.norm(v)
    return q


def umeyama(st):
    """Binary64 Umeyama per batch -> (R [B,3,3], t [B,3], q [B,4])."""
    C = st["covariance"]
    U, S, Vt = np.linalg.svd(C)
    d = np.sign(np.linalg.det(U) * np.linalg.det(Vt))
    d[d == 0] = 1
    Sfix = np.tile(np.eye(3), (C.shape[0], 1, 1))
    Sfix[:, 2, 2] = d
    R = U @ Sfix @ Vt
    R[st["n"] == 0] = np.eye(3)
    t = st["model_mean"] - np.einsum("bij,bj->bi", R, st["dataset_mean"])
    t[st["n"] == 0] = 0
    return R, t, rot_to_quat(R)


def quat_to_rot(q):
    q = np.asarray(q, np.float64)
    q = q / np.linalg.norm(q, axis=-1, keepdims=True)
    x, y, z, w = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], -2)


def rotation_angle(Ra, Rb):
    """Angle (rad) of Ra^T Rb per batch: atan2(|vee(Rd - Rd^T)| / 2, (trace - 1) / 2), which keeps
    full precision for small angles (arccos of the trace alone resolves only ~sqrt(eps))."""
    Rd = np.einsum("bji,bjk->bik", Ra, Rb)
    c = (np.trace(Rd, axis1=1, axis2=2) - 1.0) / 2.0
    v = np.stack([Rd[:, 2, 1] - Rd[:, 1, 2], Rd[:, 0, 2] - Rd[:, 2, 0], Rd[:, 1, 0] - Rd[:, 0, 1]], axis=1)
    return np.arctan2(np.linalg.norm(v, axis=1) / 2.0, c)


def loss_fd_gradients(dataset, model, gR, gt, pre=None, h=1e-6, **filt):
    """Binary64 central differences of L = <gR, R> + <gt, t> w.r.t. every dataset and model
    coordinate (small problems only).  The correspondence set is fixed at the unperturbed
    points, as the analytic backward assumes."""
    dataset = np.asarray(dataset, np.float64)
    model = np.asarray(model, np.float64)
    D0, M0, ok = correspondences(dataset.astype(F32), model.astype(F32), pre, **filt)
    if pre is not None:
        Tp = np.asarray(pre, np.float64).reshape(-1, 8)
        Rp = quat_to_rot(Tp[:, :4])
        tp = Tp[:, 4:7]
        if Rp.shape[0] == 1:
            Rp = np.broadcast_to(Rp, (dataset.shape[0], 3, 3))
            tp = np.broadcast_to(tp, (dataset.shape[0], 3))
    else:
        Rp = np.tile(np.eye(3), (dataset.shape[0], 1, 1))
        tp = np.zeros((dataset.shape[0], 3))

    def L(ds, ms):
        D = np.einsum("bij,bnj->bni", Rp, ds) + tp[:, None, :]
        st = stats(D, ms, ok)
        R, t, _ = umeyama(st)
        return (np.asarray(gR) * R).sum(axis=(1, 2)) + (np.asarray(gt) * t).sum(axis=1)

    gd = np.zeros_like(dataset)
    gm = np.zeros_like(model)
    for idx in np.ndindex(dataset.shape[1:]):
        for arr, g in ((dataset, gd), (model, gm)):
            a = arr.copy()
            b = arr.copy()
            a[(slice(None),) + idx] += h
            b[(slice(None),) + idx] -= h
            if arr is dataset:
                g[(slice(None),) + idx] = (L(a, model) - L(b, model)) / (2 * h)
            else:
                g[(slice(None),) + idx] = (L(dataset, a) - L(dataset, b)) / (2 * h)
    return gd, gm


def simulate_statistics(scene, model, Tsb, Tbm, dataset, dmask=None, dids=None, dataset_id=0, pre=None,
                        max_dist=np.inf, point_to_plane=True, fast=False):
    """The RCC / MICP-L inner step per pose (tests/embree/correction_rcc.cpp:139-160): simulate
    the model scan (Points, Normals, Hits) at Tbm[p] (oracle.Scene.simulate), pair it ray by ray
    with the dataset scan (one [W*H, 3] scan for all poses or [P, W*H, 3] per pose),
    statistics_p2l / _p2p (statistics.cpp:19-126) in binary64 and Umeyama (optimization.cpp:12-49).
    Returns (stats dict, R, t, q, per-ray validity [P, W*H]).  fast: the ray cast through the
    4-wide walk (the same outputs)."""
    Tbm = np.asarray(Tbm, F32).reshape(-1, 8)
    P = Tbm.shape[0]
    sim = scene.simulate(model, Tsb, Tbm, attrs=("hits", "points", "normals"), fast=fast)
    N = sim["hits"].size // P
    ds = np.asarray(dataset, F32).reshape(-1, N, 3)
    ds = np.broadcast_to(ds, (P, N, 3)) if ds.shape[0] == 1 else ds

    def per_pose(a):
        if a is None:
            return None
        a = np.asarray(a).reshape(-1, N)
        return np.broadcast_to(a, (P, N)) if a.shape[0] == 1 else a

    D, M, ok = correspondences(ds, sim["points"].reshape(P, N, 3), pre, dmask=per_pose(dmask),
                               mmask=sim["hits"].reshape(P, N), dids=per_pose(dids), dataset_id=dataset_id,
                               max_dist=max_dist,
                               normals=sim["normals"].reshape(P, N, 3) if point_to_plane else None)
    st = stats(D, M, ok)
    R, t, q = umeyama(st)
    return st, R, t, q, ok
