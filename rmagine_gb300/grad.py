"""Differentiable range simulation on the GB300 (range adjoint over the C ABI).

range_pose_grad() runs rmg_range_pose_grad: per pose the Huber range loss against observed
ranges and its gradient with respect to the 6-DoF right perturbation xi = (rho, omega) of the
pose (T_bm * exp(xi^)).  RangePoseLoss wraps it in a torch.autograd.Function for test harnesses:
its input is the perturbation xi [N, 6] applied to fixed poses, and its backward returns the
Lie-algebra gradient at the perturbed pose (exact at xi = 0, where the harness evaluates it).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .simulation import _Simulator


def so3_exp(w: torch.Tensor) -> torch.Tensor:
    """Rotation vector [N,3] -> unit quaternion (x, y, z, w) [N,4]."""
    th = torch.linalg.norm(w, dim=1, keepdim=True)
    half = 0.5 * th
    k = torch.where(th > 1e-12, torch.sin(half) / th.clamp_min(1e-30), 0.5 - th * th / 48.0)
    return torch.cat([w * k, torch.cos(half)], dim=1)


def perturb(Tbm: torch.Tensor, xi: torch.Tensor) -> torch.Tensor:
    """T_bm * (exp(omega^), rho): the pose moved by the right perturbation xi = (rho, omega)."""
    from .transforms import compose

    q = so3_exp(xi[:, 3:6].double()).float()
    d = torch.zeros((xi.shape[0], 8), dtype=torch.float32)
    d[:, :4] = q.cpu()
    d[:, 4:7] = xi[:, 0:3].detach().float().cpu()
    out = compose(Tbm.detach().cpu().numpy(), d.numpy())
    return torch.from_numpy(out).to(Tbm.device)


def range_pose_grad(sim: _Simulator, Tbm: torch.Tensor, ranges_obs: torch.Tensor, delta: float = 0.2,
                    want_sim: bool = False):
    """Returns (grad [N,6], loss [N]) and, with want_sim, the simulated (ranges, face_ids), on the
    device.  Observed ranges in host memory go through rmg_range_pose_grad_host instead: uploads and
    downloads in pose chunks overlap the launches, and the results come back in host memory (the
    same values as one call on device data)."""
    sim._check_ready()
    if isinstance(ranges_obs, torch.Tensor) and not ranges_obs.is_cuda:
        return _range_pose_grad_host(sim, Tbm, ranges_obs, delta, want_sim)
    Tbm = Tbm.reshape(-1, 8).to("cuda").contiguous()
    n = Tbm.shape[0]
    W, H = sim.sensor.width, sim.sensor.height
    obs = ranges_obs.reshape(-1).to("cuda", torch.float32).contiguous()
    if obs.numel() != n * W * H:
        raise L.RmgError(L.RMG_ERR_INVALID_ARG, "range_pose_grad", "ranges_obs must hold n_poses*W*H values")
    grad = torch.empty((n, 6), dtype=torch.float32, device="cuda")
    loss = torch.empty((n,), dtype=torch.float32, device="cuda")
    rs = torch.empty((n * W * H,), dtype=torch.float32, device="cuda") if want_sim else None
    fs = torch.empty((n * W * H,), dtype=torch.int32, device="cuda") if want_sim else None
    p = lambda t: None if t is None else C.c_void_p(t.data_ptr())  # noqa: E731
    L.call("rmg_range_pose_grad", sim._map.handle, sim.sensor.handle, C.byref(sim._Tsb), p(Tbm), n, p(obs),
           float(delta), p(grad), p(loss), p(rs), p(fs), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if want_sim:
        return grad, loss, rs, fs
    return grad, loss


def _range_pose_grad_host(sim, Tbm, ranges_obs, delta, want_sim):
    """Observations in host memory: rmg_range_pose_grad_host uploads them in pose chunks and
    downloads the results while other chunks are computed; the results come back in host memory
    when the call returns."""
    T = (Tbm if isinstance(Tbm, torch.Tensor) else torch.as_tensor(np.asarray(Tbm, np.float32)))
    T = T.reshape(-1, 8).to(torch.float32).contiguous()
    n = T.shape[0]
    W, H = sim.sensor.width, sim.sensor.height
    obs = torch.as_tensor(ranges_obs).reshape(-1).to(torch.float32).contiguous()
    if obs.numel() != n * W * H:
        raise L.RmgError(L.RMG_ERR_INVALID_ARG, "range_pose_grad", "ranges_obs must hold n_poses*W*H values")
    grad = torch.empty((n, 6), dtype=torch.float32)
    loss = torch.empty((n,), dtype=torch.float32)
    rs = torch.empty((n * W * H,), dtype=torch.float32) if want_sim else None
    fs = torch.empty((n * W * H,), dtype=torch.int32) if want_sim else None
    p = lambda t: None if t is None else C.c_void_p(t.data_ptr())  # noqa: E731
    L.call("rmg_range_pose_grad_host", sim._map.handle, sim.sensor.handle, C.byref(sim._Tsb), p(T), n, p(obs),
           float(delta), p(grad), p(loss), p(rs), p(fs), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if want_sim:
        return grad, loss, rs, fs
    return grad, loss


class RangePoseLoss(torch.autograd.Function):
    """loss[N] = per-pose Huber range loss at T_bm * exp(xi^); d loss / d xi from the adjoint kernel."""

    @staticmethod
    def forward(ctx, xi, sim, Tbm, ranges_obs, delta):
        T = perturb(Tbm, xi) if bool((xi != 0).any()) else Tbm.reshape(-1, 8).to("cuda")
        grad, loss = range_pose_grad(sim, T, ranges_obs, delta)
        ctx.save_for_backward(grad)
        return loss.to(xi.device)

    @staticmethod
    def backward(ctx, gloss):
        (grad,) = ctx.saved_tensors
        return (gloss.to(grad.device)[:, None] * grad).to(gloss.device), None, None, None, None
