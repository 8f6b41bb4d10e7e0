"""Shared small case of the adjoint tests: two replicas of a 2D WCA worm
system, 30-step horizon in segments of 10, and the S / C_v loss."""
from __future__ import annotations

import numpy as np
import torch

from nwgb.init import initial_state, wca_config
from nwgb.observables import PairSample, loss_s_cv

THETA0 = np.array([1.0, 10.0, 57.0, 0.5])  # eps, k_bend, k_bond, F_act
R, H, SEG = 2, 30, 10


def make_case(lib, kT=0.1):
    cfg = wca_config(24, 8, (18.0, 18.0), seed=5, lib=lib)
    cfg.kT = kT
    pos, vel = [], []
    for r in range(R):
        p, v = initial_state(cfg, seed=40 + r, layout="rows")
        pos.append(p)
        vel.append(v)
    return cfg, np.concatenate(pos), np.concatenate(vel)


def loss_fn(cfg, pos, vel, pairs, cv_target):
    """pos, vel: (N, 3) or float4 (N, 4) tensors of the final state."""
    pos = pos[:, :3].reshape(R, -1, 3)
    vel = vel[:, :3].reshape(R, -1, 3)
    box = [cfg.box[0], cfg.box[1], cfg.box[2]]
    return loss_s_cv(pos, vel, cfg.filament_size, box, pairs, cv_target)


def pairs_and_target(cfg, device="cpu"):
    pairs = PairSample(R, cfg.n_beads, 4000, seed=3, device=device)
    cv_target = torch.zeros((R, 32), dtype=torch.float64, device=device)
    return pairs, cv_target
