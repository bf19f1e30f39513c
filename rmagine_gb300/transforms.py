"""Host-side rmagine Transform arithmetic in binary32 (numpy), exact operation order.

Transform records are float32 [..., 8]: quaternion (x, y, z, w), translation (x, y, z), stamp.
  * qmul      Quaternion::mult       (math/types/Quaternion.tcc:35-42)
  * qrot      Quaternion * Vector3   (Quaternion.tcc:68-75): q (v, 0) q^-1
  * compose   Transform * Transform  (Transform.tcc:34-42)
  * inverse   Transform::inv         (Transform.tcc:24-30)
  * apply     Transform * Vector3    (Transform.tcc:56-60)
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def qmul(a, b):
    a = np.asarray(a, F32)
    b = np.asarray(b, F32)
    ax, ay, az, aw = (a[..., k] for k in range(4))
    bx, by, bz, bw = (b[..., k] for k in range(4))
    return np.stack([((aw * bx + ax * bw) + ay * bz) - az * by,
                     ((aw * by - ax * bz) + ay * bw) + az * bx,
                     ((aw * bz + ax * by) - ay * bx) + az * bw,
                     ((aw * bw - ax * bx) - ay * by) - az * bz], axis=-1).astype(F32)


def qinv(q):
    return (np.asarray(q, F32) * np.array([-1, -1, -1, 1], F32)).astype(F32)


def qrot(q, v):
    q = np.asarray(q, F32)
    v = np.asarray(v, F32)
    P = np.concatenate([v, np.zeros(v.shape[:-1] + (1,), F32)], axis=-1)
    return qmul(qmul(q, P), qinv(q))[..., :3]


def compose(T1, T2):
    T1 = np.asarray(T1, F32)
    T2 = np.asarray(T2, F32)
    out = np.zeros(np.broadcast_shapes(T1.shape, T2.shape), F32)
    rt = qrot(T1[..., :4], T2[..., 4:7])
    out[..., :4] = qmul(T1[..., :4], T2[..., :4])
    out[..., 4:7] = rt + T1[..., 4:7]
    return out


def inverse(T):
    T = np.asarray(T, F32)
    out = np.zeros_like(T)
    out[..., :4] = qinv(T[..., :4])
    out[..., 4:7] = -qrot(out[..., :4], T[..., 4:7])
    return out


def apply(T, v):
    T = np.asarray(T, F32)
    return (qrot(T[..., :4], v) + T[..., 4:7]).astype(F32)


def identity(n: int | None = None):
    t = np.array([0, 0, 0, 1, 0, 0, 0, 0], F32)
    return t if n is None else np.tile(t, (n, 1))


def to_matrix(q):
    """Unit quaternion (x, y, z, w) -> rotation matrix (binary64)."""
    q = np.asarray(q, np.float64)
    x, y, z, w = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], -2)


def yaw(q):
    """Yaw of EulerAngles from a quaternion (Quaternion.tcc:208-250 convention)."""
    q = np.asarray(q, np.float64)
    x, y, z, w = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    return np.arctan2(2.0 * (w * z + x * y), 1.0 - 2.0 * (y * y + z * z))
