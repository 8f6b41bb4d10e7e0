"""Long-run statistics: with the same initial state and seed, the GPU run and
the FP64 oracle (the reference's step restated on the CPU) separate
trajectory by trajectory (the dynamics is chaotic) but must give the same
kinetic temperature, nematic order S2 and mean-square displacement within
statistical error.  2000 steps of the 4k-bead WCA workload; temperature and
S2 sampled every 50 steps from step 500 with errors from block averages (4
blocks); the MSD at the last sample with its error across the 400 worms
(beads of one worm move together).  Compared at 4 standard errors of the
difference plus a small floor.  (The active drive keeps the kinetic
temperature above the bath's kT, in both runs alike.)"""
from __future__ import annotations

import numpy as np
import pytest

from nwgb import abi
from nwgb.init import baseline_config, initial_state

pytestmark = pytest.mark.gpu

STEPS, EVERY, BURN = 2000, 50, 500


def tangents(pos, L, box):
    r = pos[:, :2].reshape(-1, L, 2)
    nxt = np.concatenate([r[:, 1:], r[:, -1:]], 1)
    prv = np.concatenate([r[:, :1], r[:, :-1]], 1)
    d = nxt - prv
    d = np.where(d > box / 2, d - box, np.where(d < -box / 2, d + box, d))
    return d / np.linalg.norm(d, axis=-1, keepdims=True)


def observables(samples, L, box):
    """Per sample temperature and S2; per worm the final mean-square
    displacement of unwrapped positions."""
    T, S = [], []
    unwrapped = samples[0][0][:, :2].astype(np.float64).copy()
    ref = unwrapped.copy()
    prev = samples[0][0][:, :2].astype(np.float64)
    for pos, vel in samples:
        p = pos[:, :2].astype(np.float64)
        d = p - prev
        d = np.where(d > box / 2, d - box, np.where(d < -box / 2, d + box, d))
        unwrapped += d
        prev = p
        T.append((vel[:, :2].astype(np.float64) ** 2).sum(1).mean() / 2)
        t = tangents(pos.astype(np.float64), L, box)
        c = (t[..., 0] ** 2 - t[..., 1] ** 2).mean()
        s = (2 * t[..., 0] * t[..., 1]).mean()
        S.append(np.hypot(c, s))
    msd_worm = ((unwrapped - ref) ** 2).sum(1).reshape(-1, L).mean(1)
    return np.array(T), np.array(S), msd_worm


def block_stats(x, nblocks=4):
    b = np.array_split(x, nblocks)
    means = np.array([q.mean() for q in b])
    return x.mean(), means.std(ddof=1) / np.sqrt(nblocks)


def test_long_run_statistics_match_oracle(lib, orc):
    import nwgb

    cfg = baseline_config(0, seed=11)
    pos, vel = initial_state(cfg, seed=11)
    box = np.array([cfg.box[0], cfg.box[1]])
    L = cfg.filament_size
    gs = []
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.zero_forces()
        for k in range(0, STEPS, EVERY):
            s.step(EVERY, cfg.dt)
            if k + EVERY >= BURN:
                gs.append((s.get_array(abi.NW_POSITION), s.get_array(abi.NW_VELOCITY)))
        s.sync()
    z = np.zeros((cfg.n_beads, 4))
    st = dict(pos=pos.astype(np.float64), vel=vel.astype(np.float64), force=z, force_old=z, tangent=z)
    os_ = []
    for k in range(STEPS):
        st = orc.step(cfg, st, k, cfg.dt, 64)
        if (k + 1) % EVERY == 0 and k + 1 >= BURN:
            os_.append((st["pos"], st["vel"]))
    g_obs = observables(gs, L, box)
    o_obs = observables(os_, L, box)
    for name, a, b, floor in zip(("T", "S2"), g_obs[:2], o_obs[:2], (0.002, 0.01)):
        ma, ea = block_stats(a)
        mb, eb = block_stats(b)
        tol = 4.0 * np.hypot(ea, eb) + floor * max(abs(ma), abs(mb))
        assert abs(ma - mb) <= tol, (name, ma, mb, tol)
    ga, oa = g_obs[2], o_obs[2]
    sem = np.hypot(ga.std(ddof=1) / np.sqrt(ga.size), oa.std(ddof=1) / np.sqrt(oa.size))
    assert abs(ga.mean() - oa.mean()) <= 4.0 * sem + 0.02 * oa.mean(), ("MSD", ga.mean(), oa.mean(), sem)
