"""Correspondence statistics and Umeyama on the GB300 (rmagine's statistics.h / optimization.h).

Mirrors, batched:
  * statistics_p2p / statistics_p2l  (src/rmagine_core/include/rmagine/math/statistics.h:72-157,
                                      src/rmagine_cuda/include/rmagine/math/statistics.cuh:76-158)
  * umeyama_transform                 (math/optimization.h:61-75, memory_math.cuh:590-621)
  * UmeyamaReductionConstraints       (types/UmeyamaReductionConstraints.hpp:46-59)
plus the backward of p2p statistics + Umeyama.  Point clouds are float32 tensors [B, N, 3] on the
device (B batches of N correspondences); a CrossStatistics batch comes back as a float32 tensor
[B, 16] whose rows are byte-identical to rmagine::CrossStatistics (dataset_mean, model_mean,
column-major covariance, uint32 n_meas).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L


@dataclass
class UmeyamaReductionConstraints:
    max_dist: float = float("inf")
    dataset_id: int = 0
    model_id: int = 0

    def to_c(self) -> L.ConstraintsC:
        return L.ConstraintsC(self.max_dist, self.dataset_id, self.model_id)


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev(t, dtype=None):
    if t is None:
        return None
    if not isinstance(t, torch.Tensor):
        t = torch.as_tensor(np.ascontiguousarray(t))
    if dtype is not None and t.dtype != dtype:
        t = t.to(dtype)
    return t.cuda().contiguous()


def _shape(dataset):
    if dataset.dim() == 2:
        return 1, dataset.shape[0]
    return dataset.shape[0], dataset.shape[1]


def _pre(pre, B):
    if pre is None:
        return None, 0
    pre = _dev(pre, torch.float32).reshape(-1, 8)
    return pre, (1 if pre.shape[0] == B and B > 1 else 0)


def _u8(mask):
    m = _dev(mask)
    return None if m is None else m.to(torch.uint8).contiguous()


def _i32(ids):
    if ids is None:
        return None
    a = ids if isinstance(ids, torch.Tensor) else torch.as_tensor(np.asarray(ids).astype(np.uint32).view(np.int32))
    return a.to(torch.int32).cuda().contiguous()


def statistics(dataset, model, pre=None, params: UmeyamaReductionConstraints | None = None, dataset_mask=None,
               model_mask=None, dataset_ids=None, model_ids=None, model_normals=None, want_transforms=True):
    """Batched statistics_p2p (or _p2l when model_normals is given) and, optionally, the Umeyama
    transform of every batch.  Returns (stats [B,16] float32, transforms [B,8] float32 or None)."""
    params = params or UmeyamaReductionConstraints()
    dataset = _dev(dataset, torch.float32)
    model = _dev(model, torch.float32)
    B, N = _shape(dataset)
    pre_t, stride = _pre(pre, B)
    stats = torch.empty((B, 16), dtype=torch.float32, device="cuda")
    T = torch.empty((B, 8), dtype=torch.float32, device="cuda") if want_transforms else None
    dm, mm, di, mi = _u8(dataset_mask), _u8(model_mask), _i32(dataset_ids), _i32(model_ids)
    pc = params.to_c()
    lib = L.load()
    if model_normals is None:
        st = lib.rmg_statistics_p2p(_ptr(pre_t), stride, _ptr(dataset), _ptr(dm), _ptr(di), _ptr(model), _ptr(mm),
                                    _ptr(mi), C.byref(pc), B, N, _ptr(stats), _ptr(T), _stream())
        L.check(st, "rmg_statistics_p2p")
    else:
        nrm = _dev(model_normals, torch.float32)
        st = lib.rmg_statistics_p2l(_ptr(pre_t), stride, _ptr(dataset), _ptr(dm), _ptr(di), _ptr(model),
                                    _ptr(nrm), _ptr(mm), _ptr(mi), C.byref(pc), B, N, _ptr(stats), _ptr(T),
                                    _stream())
        L.check(st, "rmg_statistics_p2l")
    return stats, T


def statistics_p2p(dataset, model, pre=None, params=None, **kw):
    return statistics(dataset, model, pre, params, **kw)


def statistics_p2l(dataset, model, model_normals, pre=None, params=None, **kw):
    return statistics(dataset, model, pre, params, model_normals=model_normals, **kw)


def umeyama_transform(stats: torch.Tensor) -> torch.Tensor:
    stats = _dev(stats, torch.float32).reshape(-1, 16)
    out = torch.empty((stats.shape[0], 8), dtype=torch.float32, device="cuda")
    L.call("rmg_umeyama_transform", _ptr(stats), stats.shape[0], _ptr(out), _stream())
    return out


def svd(A, rotations: bool = False):
    """Batched 3x3 SVD A = U W V^T (rmagine's svd(As, Us, Ws, Vs), memory_math.cuh:561-578).
    A: [..., 3, 3] (row-major here; the library takes rmagine's column-major Matrix3x3).  Returns
    (U, w, V) as [..., 3, 3], [..., 3], [..., 3, 3] float32 CUDA tensors.  rotations=False: w >= 0
    sorted descending, U, V orthogonal; rotations=True: U, V rotations, w[..., 2] carries the sign of
    det A."""
    A = _dev(A, torch.float32)
    shape = A.shape[:-2]
    Acm = A.reshape(-1, 3, 3).transpose(1, 2).contiguous()  # column-major records
    n = Acm.shape[0]
    U = torch.empty((n, 3, 3), dtype=torch.float32, device="cuda")
    V = torch.empty((n, 3, 3), dtype=torch.float32, device="cuda")
    w = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    L.call("rmg_svd3", _ptr(Acm), _ptr(U), None, _ptr(w), _ptr(V), n, 1 if rotations else 0, _stream())
    return (U.transpose(1, 2).reshape(*shape, 3, 3), w.reshape(*shape, 3), V.transpose(1, 2).reshape(*shape, 3, 3))


def umeyama_backward(dataset, model, stats, grad_R=None, grad_t=None, pre=None, params=None, dataset_mask=None,
                     model_mask=None, dataset_ids=None, model_ids=None):
    """dL/d(dataset points), dL/d(model points) of L(R, t) with the given upstream gradients."""
    params = params or UmeyamaReductionConstraints()
    dataset = _dev(dataset, torch.float32)
    model = _dev(model, torch.float32)
    B, N = _shape(dataset)
    pre_t, stride = _pre(pre, B)
    gR = None if grad_R is None else _dev(grad_R, torch.float32).reshape(B, 9)
    gt = None if grad_t is None else _dev(grad_t, torch.float32).reshape(B, 3)
    gd = torch.empty_like(dataset)
    gm = torch.empty_like(model)
    dm, mm, di, mi = _u8(dataset_mask), _u8(model_mask), _i32(dataset_ids), _i32(model_ids)
    pc = params.to_c()
    L.call("rmg_umeyama_backward", _ptr(pre_t), stride, _ptr(dataset), _ptr(dm), _ptr(di), _ptr(model), _ptr(mm),
           _ptr(mi), C.byref(pc), B, N, _ptr(stats), _ptr(gR), _ptr(gt), _ptr(gd), _ptr(gm), _stream())
    return gd, gm


def decode_stats(stats: torch.Tensor) -> dict:
    """[B,16] CrossStatistics records -> numpy dict (covariance as row-major [B,3,3])."""
    s = stats.detach().cpu().numpy().reshape(-1, 16)
    cov = s[:, 6:15].reshape(-1, 3, 3).transpose(0, 2, 1)  # stored column-major
    return {"dataset_mean": s[:, 0:3].copy(), "model_mean": s[:, 3:6].copy(), "covariance": cov.copy(),
            "n": s[:, 15].copy().view(np.uint32).astype(np.int64)}
