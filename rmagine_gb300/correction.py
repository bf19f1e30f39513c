"""Pose correction on the device: rmagine's RCC / MICP-L correction loop with fused steps.

The loop of tests/embree/correction_rcc.cpp:119-170, for a batch of pose estimates at once:

    for outer in range(n_outer):
        model = simulate(Tbm_est)                     # Points, Normals, Hits at the estimate
        Tpre = I
        for inner in range(n_inner):
            stats = statistics_p2l(Tpre, dataset, model, params)
            Tpre = Tpre * umeyama_transform(stats)
        Tbm_est = Tbm_est * Tpre

Each inner step is one rmg_simulate_statistics launch (the model scan is cast again at the same
Tbm_est instead of being stored, which gives the same model), and the compositions are
rmg_transforms_compose launches, so the loop never leaves the device and never synchronises.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L
from . import statistics as S
from .simulation import _Simulator, _stream_ptr


def compose(a: torch.Tensor, b: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """out[i] = a[i] * b[i] (Transform::mult) for device Transform records [n, 8]; an operand
    with one row is repeated.  out may be a (multInplace)."""
    a = a.reshape(-1, 8)
    b = b.reshape(-1, 8)
    n = max(a.shape[0], b.shape[0])
    for x in (a, b):
        if x.shape[0] not in (1, n) or not x.is_cuda or x.dtype != torch.float32 or not x.is_contiguous():
            raise L.RmgError(L.RMG_ERR_INVALID_ARG, "compose", "operands must be contiguous float32 [n|1, 8] on the GPU")
    if out is None:
        out = torch.empty((n, 8), dtype=torch.float32, device=a.device)
    L.call("rmg_transforms_compose", C.c_void_p(a.data_ptr()), 1 if a.shape[0] == n and n > 1 else 0,
           C.c_void_p(b.data_ptr()), 1 if b.shape[0] == n and n > 1 else 0, C.c_void_p(out.data_ptr()), n,
           _stream_ptr())
    return out


def correct_rcc(sim: _Simulator, dataset_points, Tbm_est, dataset_mask=None, n_outer: int = 10,
                n_inner: int = 5, params: S.UmeyamaReductionConstraints | None = None,
                point_to_plane: bool = True) -> torch.Tensor:
    """Runs the correction loop for every estimate in Tbm_est ([n, 8] or [8]) against the
    dataset scan(s) (see _Simulator.simulate_statistics for the shapes) and returns the
    corrected estimates [n, 8] on the device."""
    Tbm = S._dev(Tbm_est, torch.float32).reshape(-1, 8).clone()
    # the scans are read n_outer * n_inner times: upload them once
    dataset_points = S._dev(dataset_points, torch.float32)
    dataset_mask = S._u8(dataset_mask)
    n = Tbm.shape[0]
    ident = torch.zeros((n, 8), dtype=torch.float32, device=Tbm.device)
    ident[:, 3] = 1.0
    Tpre = torch.empty_like(ident)
    for _ in range(n_outer):
        Tpre.copy_(ident)
        for _ in range(n_inner):
            _, T = sim.simulate_statistics(Tbm, dataset_points, dataset_mask=dataset_mask, pre=Tpre, params=params,
                                           point_to_plane=point_to_plane, want_stats=False)
            compose(Tpre, T, out=Tpre)
        compose(Tbm, Tpre, out=Tbm)
    return Tbm
