"""The FP64 torch restatement of the adjoint rollout (the reference gradient
of the CUDA adjoint): its autograd gradient agrees with FP64 central finite
differences (h = 1e-4 relative) of its own forward."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from adjoint_case import H, R, SEG, THETA0, loss_fn, make_case, pairs_and_target

torch_rollout = pytest.importorskip("torch_rollout")


def test_autograd_matches_central_differences(lib, orc):
    cfg, pos, vel = make_case(lib)
    xi = torch_rollout.noise_table(cfg, R, H)
    pairs, target = pairs_and_target(cfg)

    def L(theta):
        r, v = torch_rollout.rollout(cfg, theta, pos, vel, R, H, SEG, xi)
        return loss_fn(cfg, r, v, pairs, target)

    th = torch.tensor(THETA0, dtype=torch.float64, requires_grad=True)
    L(th).backward()
    g = th.grad.numpy()
    fd = np.zeros(4)
    with torch.no_grad():
        for k in range(4):
            h = 1e-4 * THETA0[k]
            tp, tm = THETA0.copy(), THETA0.copy()
            tp[k] += h
            tm[k] -= h
            fd[k] = (L(torch.tensor(tp)).item() - L(torch.tensor(tm)).item()) / (2 * h)
    scale = np.abs(fd).max()
    assert np.all(np.abs(g - fd) <= 1e-4 * scale + 1e-6 * np.abs(fd)), (g, fd)


def test_rollout_forward_matches_oracle_step_over_a_segment(lib, orc):
    """Within one segment the frozen list holds every pair that comes within
    the cut-off, so the restatement's forward is the oracle's own FP64 step
    (oracle.step, pinned to the reference's kernels) with the same noise:
    update m of the rollout is oracle step m - 1 of replica r (seed + r)."""
    cfg, pos, vel = make_case(lib)
    n_steps = SEG
    xi = torch_rollout.noise_table(cfg, R, n_steps)
    r, v = torch_rollout.rollout(cfg, torch.tensor(THETA0, dtype=torch.float64), pos, vel, R, n_steps, n_steps, xi)
    nb = cfg.n_beads
    for rep in range(R):
        c = cfg.copy()
        c.seed = cfg.seed + rep
        z = np.zeros((nb, 4))
        st = dict(pos=pos[rep * nb:(rep + 1) * nb].astype(np.float64), vel=vel[rep * nb:(rep + 1) * nb].astype(np.float64),
                  force=z, force_old=z, tangent=z)
        for k in range(n_steps):
            st = orc.step(c, st, k, c.dt, 64)
        got_r = r.detach().numpy()[rep * nb:(rep + 1) * nb]
        got_v = v.detach().numpy()[rep * nb:(rep + 1) * nb]
        assert np.abs(got_r - st["pos"][:, :3]).max() < 1e-11
        assert np.abs(got_v - st["vel"][:, :3]).max() < 1e-11 * max(1.0, np.abs(st["vel"]).max())
