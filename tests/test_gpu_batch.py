"""Batched replicas against single systems: each replica of a batch follows
the same trajectory as a single-system handle with its configuration (same
strategy, same launch-independent arithmetic) up to the order of FP32 sums,
and the batch reports its launches, tuning and errors."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err
from nwgb import abi
from nwgb.init import batch_configs, initial_state

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


@pytest.mark.parametrize("strategy", [abi.NW_STRATEGY_VERLET, abi.NW_STRATEGY_CELL_LISTS])
@pytest.mark.parametrize("threads", [128, 256, 512])
def test_batch_matches_single_systems(lib, strategy, threads):
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
            assert rel_err(b.get_array(r, abi.NW_POSITION), p) < 1e-5, r
            assert rel_err(b.get_array(r, abi.NW_VELOCITY), v) < 1e-4, r
            assert rel_err(b.get_array(r, abi.NW_FORCE), f) < 1e-3, r


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
        assert t.ms_per_step > 0
        assert b.step_index == 3
        for r in range(len(cfgs)):
            assert np.array_equal(b.get_array(r, abi.NW_POSITION), before[r])
        b.step(5)
        b.sync()


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
