"""ORACLE -- test infrastructure only.  Binary64 host reference of the range adjoint.

For each ray with a given hit face (from the simulation under test) it re-intersects the
face's plane in binary64 for the pose T_bm * (exp(omega^), rho):
    r(xi) = n . (p0 - o(xi)) / (n . d(xi))
and forms per pose
  * the analytic gradient  sum psi(r - r_obs) dr/dxi, dr/drho = -n_b / (n_b.d_b),
    dr/domega = -(p_b x n_b) / (n_b.d_b)  (base-frame quantities, as documented in the library);
  * central finite differences of sum Huber(r(xi) - r_obs) with step h on the rays whose hit
    stays inside the same triangle at every +-h sample (stable face).
Pose math follows rmagine (Transform.tcc:34-42: sensor in map = T_bm * T_sb).
"""
from __future__ import annotations

import numpy as np


def quat_to_rot(q):
    q = np.asarray(q, np.float64)
    x, y, z, w = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], -2)


def rodrigues(w):
    w = np.asarray(w, np.float64)
    th = np.linalg.norm(w, axis=-1, keepdims=True)
    k = np.where(th > 0, w / np.where(th > 0, th, 1), 0)
    K = np.zeros(w.shape[:-1] + (3, 3))
    K[..., 0, 1], K[..., 0, 2] = -k[..., 2], k[..., 1]
    K[..., 1, 0], K[..., 1, 2] = k[..., 2], -k[..., 0]
    K[..., 2, 0], K[..., 2, 1] = -k[..., 1], k[..., 0]
    s, c = np.sin(th)[..., None], np.cos(th)[..., None]
    return np.eye(3) + s * K + (1 - c) * (K @ K)


def huber(e, delta):
    a = np.abs(e)
    return np.where(a <= delta, 0.5 * e * e, delta * (a - 0.5 * delta))


class RayFaceSet:
    """Rays (pose index, sensor-frame direction/origin) with their fixed hit faces."""

    def __init__(self, vertices, faces, Tsb, Tbm, dirs_s, origs_s, pose_idx, face_idx, r_obs):
        v = np.asarray(vertices, np.float64)
        f = np.asarray(faces, np.int64)[np.asarray(face_idx, np.int64)]
        self.p0, self.p1, self.p2 = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
        self.n = np.cross(self.p1 - self.p0, self.p2 - self.p0)
        Tsb = np.asarray(Tsb, np.float64).reshape(8)
        Rsb = quat_to_rot(Tsb[:4])
        self.db = np.asarray(dirs_s, np.float64) @ Rsb.T
        self.ob = Tsb[4:7] + np.asarray(origs_s, np.float64) @ Rsb.T
        T = np.asarray(Tbm, np.float64).reshape(-1, 8)[np.asarray(pose_idx)]
        self.Rbm = quat_to_rot(T[:, :4])
        self.tbm = T[:, 4:7]
        self.pose = np.asarray(pose_idx)
        self.obs = np.asarray(r_obs, np.float64)

    def ranges(self, rho=None, omega=None):
        """r for each ray at T_bm * (exp(omega^), rho) (per-ray rho/omega [M,3] or None)."""
        ob, db = self.ob, self.db
        if omega is not None:
            Rw = rodrigues(omega)
            ob = np.einsum("mij,mj->mi", Rw, ob)
            db = np.einsum("mij,mj->mi", Rw, db)
        if rho is not None:
            ob = ob + rho
        o = np.einsum("mij,mj->mi", self.Rbm, ob) + self.tbm
        d = np.einsum("mij,mj->mi", self.Rbm, db)
        return np.einsum("mi,mi->m", self.n, self.p0 - o) / np.einsum("mi,mi->m", self.n, d), o, d

    def inside(self, o, d, r):
        p = o + r[:, None] * d
        e0, e1, e2 = self.p1 - self.p0, self.p2 - self.p0, p - self.p0
        d00, d01, d11 = (e0 * e0).sum(1), (e0 * e1).sum(1), (e1 * e1).sum(1)
        d20, d21 = (e2 * e0).sum(1), (e2 * e1).sum(1)
        den = d00 * d11 - d01 * d01
        v = (d11 * d20 - d01 * d21) / den
        w = (d00 * d21 - d01 * d20) / den
        return np.minimum(np.minimum(v, w), 1 - v - w)

    def analytic(self, n_poses, delta):
        r, o, d = self.ranges()
        psi = np.clip(r - self.obs, -delta, delta)
        nb = np.einsum("mji,mj->mi", self.Rbm, self.n)  # R_bm^T n
        b = np.einsum("mi,mi->m", nb, self.db)
        pb = self.ob + r[:, None] * self.db
        g = np.concatenate([-nb / b[:, None], -np.cross(pb, nb) / b[:, None]], axis=1) * psi[:, None]
        out = np.zeros((n_poses, 6))
        np.add.at(out, self.pose, g)
        loss = np.zeros(n_poses)
        np.add.at(loss, self.pose, huber(r - self.obs, delta))
        return out, loss

    def finite_differences(self, n_poses, delta, h=1e-4, band=1e-9):
        """Central differences on stable rays; returns (fd [P,6], analytic on the same rays [P,6], stable mask)."""
        M = self.obs.size
        stable = np.ones(M, bool)
        vals = []
        for k in range(6):
            pair = []
            for sgn in (1.0, -1.0):
                step = np.zeros((M, 3))
                step[:, k % 3] = sgn * h
                r, o, d = self.ranges(rho=step if k < 3 else None, omega=step if k >= 3 else None)
                stable &= self.inside(o, d, r) > band
                pair.append(r)
            vals.append(pair)
        fd = np.zeros((n_poses, 6))
        for k in range(6):
            lp = huber(vals[k][0] - self.obs, delta) * stable
            lm = huber(vals[k][1] - self.obs, delta) * stable
            np.add.at(fd[:, k], self.pose, (lp - lm) / (2 * h))
        r, o, d = self.ranges()
        psi = np.clip(r - self.obs, -delta, delta) * stable
        nb = np.einsum("mji,mj->mi", self.Rbm, self.n)
        b = np.einsum("mi,mi->m", nb, self.db)
        pb = self.ob + r[:, None] * self.db
        g = np.concatenate([-nb / b[:, None], -np.cross(pb, nb) / b[:, None]], axis=1) * psi[:, None]
        an = np.zeros((n_poses, 6))
        np.add.at(an, self.pose, g)
        return fd, an, stable
