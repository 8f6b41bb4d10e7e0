"""The CUDA adjoint rollout against the FP64 reference gradient (torch
autograd through oracle/torch_rollout.py) and against central finite
differences of its own FP64 forward, on two replicas of a 2D WCA worm system
over 30 steps with lists frozen per 10-step segment.  Tolerances: 1e-4 of
the largest gradient component (the bar for dL/d(eps, k_bend, k_bond,
F_act)) in FP64; FP32 states and arithmetic stay within 1e-3.  The rollout
returns float4 arrays at either precision, so final positions agree with
the FP64 reference to FP32 rounding (|x| < 10: 1e-6), and the finite
differences of its own forward use h = 1e-3 of each parameter, large
enough that the FP32 rounding of the outputs does not enter (the FP64
h = 1e-4 check of the reference itself is in test_adjoint_reference.py)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from adjoint_case import H, R, SEG, THETA0, loss_fn, make_case, pairs_and_target

pytestmark = pytest.mark.gpu
torch_rollout = pytest.importorskip("torch_rollout")


@pytest.fixture(scope="module")
def case(lib, orc):
    cfg, pos, vel = make_case(lib)
    xi = torch_rollout.noise_table(cfg, R, H)
    pairs, target = pairs_and_target(cfg)
    th = torch.tensor(THETA0, dtype=torch.float64, requires_grad=True)
    r, v = torch_rollout.rollout(cfg, th, pos, vel, R, H, SEG, xi)
    L = loss_fn(cfg, r, v, pairs, target)
    L.backward()
    return cfg, pos, vel, r.detach().numpy(), th.grad.numpy(), L.item()


def gpu_grad(cfg, pos, vel, precision):
    from nwgb.adjoint import Rollout, rollout

    ro = Rollout(cfg, R, H, SEG, precision)
    ro.set_state(torch.from_numpy(pos).cuda(), torch.from_numpy(vel).cuda())
    pairs, target = pairs_and_target(cfg, device="cuda")
    th = torch.tensor(THETA0, dtype=torch.float64, requires_grad=True)
    p, v = rollout(th, ro)
    L = loss_fn(cfg, p.double(), v.double(), pairs, target)
    L.backward()
    return ro, p.detach(), th.grad.numpy(), L.item(), pairs, target


@pytest.mark.parametrize("precision,tol", [(64, 1e-4), (32, 1e-3)])
def test_adjoint_matches_fp64_reference_gradient(case, precision, tol):
    cfg, pos, vel, r_ref, g_ref, L_ref = case
    ro, p, g, L, _, _ = gpu_grad(cfg, pos, vel, precision)
    # same final state as the FP64 reference (positions wrapped the same way)
    assert np.abs(p[:, :3].cpu().numpy() - r_ref).max() < (2e-6 if precision == 64 else 1e-4)
    assert abs(L - L_ref) <= tol * abs(L_ref)
    assert np.all(np.abs(g - g_ref) <= tol * np.abs(g_ref).max()), (g, g_ref)
    ro.close()


def test_adjoint_matches_central_differences_of_its_forward(case):
    cfg, pos, vel, _, _, _ = case
    ro, _, g, _, pairs, target = gpu_grad(cfg, pos, vel, 64)
    fd = np.zeros(4)
    with torch.no_grad():
        for k in range(4):
            h = 1e-3 * THETA0[k]
            vals = []
            for sgn in (1, -1):
                th = THETA0.copy()
                th[k] += sgn * h
                p, v = ro.forward(th)
                vals.append(loss_fn(cfg, p.double(), v.double(), pairs, target).item())
            fd[k] = (vals[0] - vals[1]) / (2 * h)
    assert np.all(np.abs(g - fd) <= 1e-4 * np.abs(fd).max()), (g, fd)
    ro.close()


def test_rollout_is_deterministic_and_reports_timings(case):
    cfg, pos, vel, _, _, _ = case
    ro1, p1, g1, _, _, _ = gpu_grad(cfg, pos, vel, 32)
    ro2, p2, g2, _, _, _ = gpu_grad(cfg, pos, vel, 32)
    assert torch.equal(p1, p2)
    assert np.array_equal(g1, g2)
    f_ms, b_ms = ro1.timings()
    assert f_ms > 0 and b_ms > 0
    ro1.close()
    ro2.close()
