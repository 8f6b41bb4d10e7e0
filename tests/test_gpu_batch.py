"""Batched replicas: every replica of a batch against the oracle's step of
its own configuration, per bead (tests/parity.py); against a single-system
handle of the same configuration over a trajectory (same strategy, up to the
order of FP32 sums); launches, tuning and errors."""
from __future__ import annotations

import numpy as np
import pytest

from nwgb import abi
from nwgb.init import batch_configs, initial_state
from parity import TOL, force_err, fp64_bound, update_err, vec_err

pytestmark = pytest.mark.gpu


def small_batch(lib, n=6, seed=3):
    cfgs = batch_configs(n, seed=seed, lib=lib, worms=(20, 120), beads=(5, 30))
    states = [initial_state(c, seed=100 + r, layout="rows") for r, c in enumerate(cfgs)]
    return cfgs, states


def run_single(cfg, pos, vel, nsteps, strategy):
    import nwgb

    cfg.strategy = strategy
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.step(nsteps, cfg.dt)
        s.sync()
        return s.get_array(abi.NW_POSITION), s.get_array(abi.NW_VELOCITY), s.get_array(abi.NW_FORCE)


def periodic_box(cfg):
    return np.array([cfg.box[a] if cfg.boundary[a] == abi.NW_PERIODIC else 0.0 for a in range(3)])


@pytest.mark.parametrize("strategy", [abi.NW_STRATEGY_VERLET, abi.NW_STRATEGY_CELL_LISTS])
def test_batch_replicas_match_oracle(lib, orc, strategy):
    """One step of every replica of an uneven batch (worm counts, lengths,
    F_act, k_bend, boxes differ) from a state with non-zero forces, against
    the FP32 and FP64 oracle steps of that replica's configuration: forces
    per bead within 1e-5 of the force scale, velocities relative, positions
    relative to the displacement."""
    import nwgb

    cfgs, states = small_batch(lib, n=7, seed=13)
    starts = []
    for r, (c, (pos, vel)) in enumerate(zip(cfgs, states)):
        z = np.zeros((c.n_beads, 4), np.float32)
        s1 = orc.step(c, dict(pos=pos, vel=vel, force=z, force_old=z, tangent=z), 0, c.dt, 32)
        starts.append(s1)
    with nwgb.Batch(cfgs) as b:
        b.set_tuning(256, strategy, 0.3)
        for r, s1 in enumerate(starts):
            b.set_array(r, abi.NW_POSITION, s1["pos"])
            b.set_array(r, abi.NW_VELOCITY, s1["vel"])
            b.set_array(r, abi.NW_FORCE, s1["force"])
            b.set_array(r, abi.NW_FORCE_OLD, s1["force_old"])
        b.step(1)
        b.sync()
        got = [{k: b.get_array(r, a) for k, a in (("pos", abi.NW_POSITION), ("vel", abi.NW_VELOCITY),
                                                   ("force", abi.NW_FORCE), ("force_old", abi.NW_FORCE_OLD))}
               for r in range(len(cfgs))]
    for r, (c, s1, g) in enumerate(zip(cfgs, starts, got)):
        st = {k: s1[k] for k in ("pos", "vel", "force", "force_old", "tangent")}
        o = orc.step(c, st, 0, c.dt, 32)
        o64 = orc.step(c, st, 0, c.dt, 64, force_scale=True)
        assert np.array_equal(g["force_old"][:, :3], s1["force"][:, :3]), r
        S, box = o64["force_scale"], periodic_box(c)
        for m in (lambda x, y: force_err(x["force"], y["force"], S),
                  lambda x, y: vec_err(x["vel"], y["vel"]),
                  lambda x, y: update_err(x["pos"], y["pos"], s1["pos"], box)):
            assert m(g, o) < TOL, r
            assert m(g, o64) < fp64_bound(m(o, o64)), r


@pytest.mark.parametrize("strategy", [abi.NW_STRATEGY_VERLET, abi.NW_STRATEGY_CELL_LISTS])
@pytest.mark.parametrize("threads", [128, 256, 512])
def test_batch_matches_single_systems(lib, orc, strategy, threads):
    import nwgb

    cfgs, states = small_batch(lib)
    n = 25
    with nwgb.Batch(cfgs) as b:
        b.set_tuning(threads, strategy, 0.3)
        for r, (pos, vel) in enumerate(states):
            b.set_array(r, abi.NW_POSITION, pos)
            b.set_array(r, abi.NW_VELOCITY, vel)
        b.step(n)
        b.sync()
        assert b.step_index == n
        # pro, (n - 1) fused, epi, step counter; Verlet batches add a list kernel after each pro part
        assert b.last_launch_count == (2 * n + 2 if strategy == abi.NW_STRATEGY_VERLET else n + 2)
        for r, c in enumerate(cfgs):
            c.neighbor_skin = 0.3
            p, v, f = run_single(c, *states[r], n, strategy)
            # 25 steps apart from any common state: per-bead differences are
            # FP32 summation-order differences grown along the trajectory
            z = np.zeros((c.n_beads, 4), np.float32)
            st = dict(pos=states[r][0], vel=states[r][1], force=z, force_old=z, tangent=z)
            for k in range(n):
                st = orc.step(c, st, k, c.dt, 64, force_scale=k == n - 1)
            assert update_err(b.get_array(r, abi.NW_POSITION), p, states[r][0], periodic_box(c)) < 1e-4, r
            assert vec_err(b.get_array(r, abi.NW_VELOCITY), v) < 1e-4, r
            assert force_err(b.get_array(r, abi.NW_FORCE), f, st["force_scale"]) < 1e-4, r


def test_batch_graph_replay_is_deterministic(lib):
    import nwgb

    cfgs, states = small_batch(lib, n=4, seed=7)
    out = []
    for graphs in (True, False, True):
        with nwgb.Batch(cfgs) as b:
            b.set_graphs(graphs)
            for r, (pos, vel) in enumerate(states):
                b.set_array(r, abi.NW_POSITION, pos)
                b.set_array(r, abi.NW_VELOCITY, vel)
            b.step(10)
            b.step(10)
            b.sync()
            out.append([b.get_array(r, abi.NW_POSITION) for r in range(len(cfgs))])
    for r in range(len(cfgs)):
        assert np.array_equal(out[0][r], out[1][r])
        assert np.array_equal(out[0][r], out[2][r])


def test_autotune_keeps_state_and_picks_a_candidate(lib):
    import nwgb

    cfgs, states = small_batch(lib, n=5, seed=11)
    with nwgb.Batch(cfgs) as b:
        for r, (pos, vel) in enumerate(states):
            b.set_array(r, abi.NW_POSITION, pos)
            b.set_array(r, abi.NW_VELOCITY, vel)
        b.step(3)
        b.sync()
        before = [b.get_array(r, abi.NW_POSITION) for r in range(len(cfgs))]
        t = b.autotune(trial_steps=5)
        assert t.threads_per_block in (128, 256, 512)
        assert t.strategy in (abi.NW_STRATEGY_VERLET, abi.NW_STRATEGY_CELL_LISTS)
        assert t.cell_capacity in (8, 16)
        assert t.ms_per_step > 0
        assert b.step_index == 3
        for r in range(len(cfgs)):
            assert np.array_equal(b.get_array(r, abi.NW_POSITION), before[r])
        b.step(5)
        b.sync()
        key = b.tuning_class
    # a batch of the same class takes the cached tuning without timing
    with nwgb.Batch(cfgs) as b2:
        assert b2.tuning_class == key
        t2 = b2.autotune(trial_steps=0)
        assert (t2.threads_per_block, t2.strategy, t2.cell_capacity) == (t.threads_per_block, t.strategy,
                                                                           t.cell_capacity)
        assert t2.neighbor_skin == t.neighbor_skin and t2.ms_per_step == t.ms_per_step


def test_tuning_cell_capacity(lib):
    """Slots per list cell as a tuning axis: 8 and 16 give the same
    trajectory (no cell overflows here); other values are rejected."""
    import nwgb

    cfgs, states = small_batch(lib, n=3, seed=4)
    out = []
    for cap in (8, 16):
        with nwgb.Batch(cfgs) as b:
            b.set_tuning(256, abi.NW_STRATEGY_VERLET, 0.3, cap)
            assert b.tuning.cell_capacity == cap
            for r, (pos, vel) in enumerate(states):
                b.set_array(r, abi.NW_POSITION, pos)
                b.set_array(r, abi.NW_VELOCITY, vel)
            b.step(10)
            b.sync()
            out.append([b.get_array(r, abi.NW_POSITION) for r in range(len(cfgs))])
            with pytest.raises(nwgb.NwError) as e:
                b.set_tuning(256, abi.NW_STRATEGY_VERLET, 0.3, 12)
            assert e.value.status == abi.NW_ERR_INVALID
    for r in range(len(cfgs)):
        assert np.array_equal(out[0][r], out[1][r])


def test_batch_rejects_solvent_and_reports_nonfinite(lib):
    import nwgb
    from nwgb.init import wca_config

    c = wca_config(10, 10, (20.0, 20.0), srd=True, lib=lib)
    with pytest.raises(nwgb.NwError) as e:
        nwgb.Batch([c])
    assert e.value.status == abi.NW_ERR_UNSUPPORTED
    cfgs, states = small_batch(lib, n=3, seed=5)
    with nwgb.Batch(cfgs) as b:
        for r, (pos, vel) in enumerate(states):
            p = pos.copy()
            if r == 1:
                p[3, 0] = np.nan
            b.set_array(r, abi.NW_POSITION, p)
            b.set_array(r, abi.NW_VELOCITY, vel)
        b.step(2)
        with pytest.raises(nwgb.NwError) as e:
            b.sync()
        assert e.value.status == abi.NW_ERR_NONFINITE
