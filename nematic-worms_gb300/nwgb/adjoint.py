"""Differentiable rollout (include/nwgb_adjoint.h) as a torch.autograd.Function.

    ro = Rollout(cfg, n_replicas=64, horizon=200, segment=20)
    ro.set_state(pos0, vel0)                   # float4 CUDA tensors (R * nb, 4)
    theta = torch.tensor([eps, k_bend, k_bond, F_act], dtype=torch.float64, requires_grad=True)
    pos, vel = rollout(theta, ro)              # final state, float32 CUDA
    loss = f(pos, vel); loss.backward()        # theta.grad from the CUDA adjoint

The forward runs on the CUDA engine with a fixed noise realisation and
neighbour lists frozen per segment; the backward runs the hand-written
adjoint kernels (checkpoints every `segment` steps, recomputed in between).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import abi
from .abi import NwConfig, check


class Rollout:
    """One nw_adjoint handle: n_replicas copies of cfg, seeds cfg.seed + r."""

    def __init__(self, cfg: NwConfig, n_replicas: int, horizon: int = 200, segment: int = 20, precision: int = 32,
                 lib: C.CDLL | None = None):
        self.lib = lib or abi.load_library()
        h = C.c_void_p()
        check(self.lib.nw_adj_create(C.byref(cfg), n_replicas, horizon, segment, precision, C.byref(h)),
              "nw_adj_create")
        self.h = h
        self.cfg = cfg
        self.n_replicas = n_replicas
        self.n = cfg.n_beads * n_replicas

    def close(self) -> None:
        if self.h:
            self.lib.nw_adj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _stream(self) -> None:
        check(self.lib.nw_adj_set_stream(self.h, C.c_void_p(torch.cuda.current_stream().cuda_stream)))

    def set_state(self, pos: torch.Tensor, vel: torch.Tensor) -> None:
        pos = pos.detach().to(device="cuda", dtype=torch.float32).contiguous()
        vel = vel.detach().to(device="cuda", dtype=torch.float32).contiguous()
        assert pos.shape == (self.n, 4) and vel.shape == (self.n, 4)
        self._stream()
        check(self.lib.nw_adj_set_state(self.h, C.c_void_p(pos.data_ptr()), C.c_void_p(vel.data_ptr())),
              "nw_adj_set_state")

    def forward(self, theta) -> tuple[torch.Tensor, torch.Tensor]:
        th = (C.c_double * 4)(*[float(x) for x in theta])
        pos = torch.empty((self.n, 4), dtype=torch.float32, device="cuda")
        vel = torch.empty((self.n, 4), dtype=torch.float32, device="cuda")
        self._stream()
        check(self.lib.nw_adj_forward(self.h, th, C.c_void_p(pos.data_ptr()), C.c_void_p(vel.data_ptr())),
              "nw_adj_forward")
        return pos, vel

    def final_state_f64(self) -> tuple[torch.Tensor, torch.Tensor]:
        """Final (positions, velocities) of the last forward, (n, 4) float64
        CUDA tensors (w = 0), unrounded at precision 64."""
        pos = torch.empty((self.n, 4), dtype=torch.float64, device="cuda")
        vel = torch.empty((self.n, 4), dtype=torch.float64, device="cuda")
        self._stream()
        check(self.lib.nw_adj_final_state_f64(self.h, C.c_void_p(pos.data_ptr()), C.c_void_p(vel.data_ptr())),
              "nw_adj_final_state_f64")
        return pos, vel

    def backward(self, grad_pos: torch.Tensor, grad_vel: torch.Tensor) -> np.ndarray:
        gp = grad_pos.detach().to(device="cuda", dtype=torch.float32).contiguous()
        gv = grad_vel.detach().to(device="cuda", dtype=torch.float32).contiguous()
        out = (C.c_double * 4)()
        self._stream()
        check(self.lib.nw_adj_backward(self.h, C.c_void_p(gp.data_ptr()), C.c_void_p(gv.data_ptr()), out),
              "nw_adj_backward")
        return np.array(list(out))

    def timings(self) -> tuple[float, float]:
        f, b = C.c_float(), C.c_float()
        check(self.lib.nw_adj_timings(self.h, C.byref(f), C.byref(b)))
        return f.value, b.value


class _RolloutFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta: torch.Tensor, ro: Rollout):
        pos, vel = ro.forward(theta.detach().cpu().double().numpy())
        ctx.ro = ro
        ctx.theta_meta = (theta.dtype, theta.device)
        return pos, vel

    @staticmethod
    def backward(ctx, grad_pos, grad_vel):
        ro = ctx.ro
        if grad_pos is None:
            grad_pos = torch.zeros((ro.n, 4), dtype=torch.float32, device="cuda")
        if grad_vel is None:
            grad_vel = torch.zeros((ro.n, 4), dtype=torch.float32, device="cuda")
        g = ro.backward(grad_pos, grad_vel)
        dtype, device = ctx.theta_meta
        return torch.tensor(g, dtype=dtype, device=device), None


def rollout(theta: torch.Tensor, ro: Rollout):
    """Final (positions, velocities) of ro's horizon as a function of theta =
    (eps, k_bend, k_bond, F_act), differentiable through the CUDA adjoint."""
    return _RolloutFn.apply(theta, ro)
