"""The CUDA adjoint rollout against the FP64 reference gradient (torch
autograd through oracle/torch_rollout.py) and against central finite
differences of its own FP64 forward: on two replicas of a 2D WCA worm system
over 30 steps with lists frozen per 10-step segment, and on the 64 x 4,000-
bead workload over 200 steps with 20-step segments.  Tolerances: per
parameter 1e-4 of its own gradient in FP64 (the bar for dL/d(eps, k_bend,
k_bond, F_act)); FP32 states and arithmetic stay within 1e-3 on the small
case.  Finite differences read the FP64 final state unrounded
(nw_adj_final_state_f64)."""
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
    """FP64 adjoint against FP64 central differences (h = 1e-4 of each
    parameter) of its own forward, read unrounded (nw_adj_final_state_f64),
    every parameter within 1e-4 of its own value."""
    cfg, pos, vel, _, _, _ = case
    ro, _, g, _, pairs, target = gpu_grad(cfg, pos, vel, 64)
    fd = np.zeros(4)
    with torch.no_grad():
        for k in range(4):
            h = 1e-4 * THETA0[k]
            vals = []
            for sgn in (1, -1):
                th = THETA0.copy()
                th[k] += sgn * h
                ro.forward(th)
                p, v = ro.final_state_f64()
                vals.append(loss_fn(cfg, p, v, pairs, target).item())
            fd[k] = (vals[0] - vals[1]) / (2 * h)
    assert np.all(np.abs(g - fd) <= 1e-4 * np.abs(fd)), (g, fd)
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


# ---- the 64 x 4,000-bead workload at its stated horizon ------------------------

R4, H4, SEG4 = 64, 200, 20
THETA4 = np.array([1.1, 8.0, 50.0, 0.8])  # off the reference parameters (1, 10, 57, 0.5)


@pytest.fixture(scope="module")
def workload4(lib):
    """64 replicas of the 4,000-bead workload (100 x 100 box), 200 steps with
    lists frozen per 20-step segment; C_target from a run at the reference
    parameters; the loss with its C1 bin weights (nwgb.observables)."""
    from nwgb.adjoint import Rollout
    from nwgb.init import baseline_config, initial_state
    from nwgb.observables import PairSample, velocity_correlation

    cfg = baseline_config(0, seed=7, lib=lib)
    states = [initial_state(cfg, seed=r, layout="patches") for r in range(R4)]
    pos = torch.from_numpy(np.concatenate([s[0] for s in states])).cuda()
    vel = torch.from_numpy(np.concatenate([s[1] for s in states])).cuda()
    box = [cfg.box[0], cfg.box[1], cfg.box[2]]
    pairs = PairSample(R4, cfg.n_beads, 20000, seed=1, device="cuda")
    ro = {p: Rollout(cfg, R4, H4, SEG4, p, lib) for p in (32, 64)}
    for r in ro.values():
        r.set_state(pos, vel)
    with torch.no_grad():
        ro[64].forward([1.0, 10.0, 57.0, 0.5])
        p, v = ro[64].final_state_f64()
        target = velocity_correlation(p[:, :3].reshape(R4, -1, 3), v[:, :3].reshape(R4, -1, 3), pairs,
                                      box).mean(0, keepdim=True)

    def loss(p, v):
        from nwgb.observables import loss_s_cv

        return loss_s_cv(p[:, :3].reshape(R4, -1, 3).double(), v[:, :3].reshape(R4, -1, 3).double(),
                         cfg.filament_size, box, pairs, target)

    yield cfg, ro, loss
    for r in ro.values():
        r.close()


def adjoint_gradient(ro, loss, theta):
    p, v = ro.forward(theta)
    p = p.clone().requires_grad_(True)
    v = v.clone().requires_grad_(True)
    gp, gv = torch.autograd.grad(loss(p, v), (p, v))
    assert torch.isfinite(gp).all() and torch.isfinite(gv).all()
    return ro.backward(gp, gv)


def central_differences(ro, loss, theta, hrel):
    fd = np.zeros(4)
    with torch.no_grad():
        for k in range(4):
            h = hrel * theta[k]
            vals = []
            for sgn in (1, -1):
                th = theta.copy()
                th[k] += sgn * h
                ro.forward(th)
                vals.append(loss(*ro.final_state_f64()).item())
            fd[k] = (vals[0] - vals[1]) / (2 * h)
    return fd


def test_workload4_adjoint_matches_fp64_central_differences(workload4):
    """dL/d(eps, k_bend, k_bond, F_act) of the 64 x 4,000-bead, 200-step
    rollout against FP64 central differences of the FP64 forward read
    unrounded.

    The WCA force is cut where it reaches zero but not its slope, so each of
    the many pairs that cross the cut-off during 200 steps puts a small kink
    into the loss as a function of theta: differences over h = 1e-4 of a
    parameter straddle kinks and differ from the derivative by ~1e-3 for eps
    (measured: 1.3e-3 for eps, 2.3e-4 for k_bend, < 5e-5 for k_bond and
    F_act); over h = 1e-6 they converge to it.  So: the FP64 adjoint within
    1e-4 of the h = 1e-6 differences for every parameter on its own, and
    within the h = 1e-4 differences' own spread (their change from h = 1e-4
    to 1e-6) plus 1e-4.  The FP32 adjoint is the exact gradient of the FP32
    forward, whose rounding grows along 200 steps: per parameter within its
    distance from the FP64 adjoint (measured against the h = 1e-6
    differences: 2.9e-3 for eps, 2.6e-3 for k_bend, 2e-5 for k_bond, 2.7e-5
    for F_act; 1.2e-4 of the largest component), bounded here at 2e-4 of the
    largest component."""
    cfg, ro, loss = workload4
    g64 = adjoint_gradient(ro[64], loss, THETA4)
    g32 = adjoint_gradient(ro[32], loss, THETA4)
    assert np.all(np.isfinite(g64)) and np.all(np.isfinite(g32)), (g64, g32)
    fd4 = central_differences(ro[64], loss, THETA4, 1e-4)
    fd6 = central_differences(ro[64], loss, THETA4, 1e-6)
    assert np.all(np.abs(g64 - fd6) <= 1e-4 * np.abs(fd6)), (g64, fd6, np.abs(g64 - fd6) / np.abs(fd6))
    assert np.all(np.abs(g64 - fd4) <= 2.0 * np.abs(fd4 - fd6) + 1e-4 * np.abs(fd4)), (g64, fd4, fd6)
    assert np.all(np.abs(g32 - fd6) <= 2e-4 * np.abs(fd6).max()), (g32, fd6)
    assert np.all(np.abs(g32 - fd6) <= 1.5 * np.abs(g32 - g64) + 1e-4 * np.abs(fd6)), (g32, g64, fd6)
