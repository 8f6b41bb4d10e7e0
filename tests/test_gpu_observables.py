"""Observables on the device (nw_observe, nw_velocity_correlation,
nw_srd_temperature_histogram) against the numpy oracle
(oracle/observables_oracle.py, pinned to the reference's analysis by
tests/test_observables.py).

Tolerances: order parameters 1e-6 (device tangents rounded to float32 from
double, the oracle's in float32 arithmetic), temperatures and mean-square
displacement 1e-12 relative (double sums in another order), pair sums 1e-10
relative, the SRD histogram exactly (fixed-point cell sums on both sides)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN
from nwgb import abi
from nwgb.init import initial_state, wca_config

import observables_oracle as obs

pytestmark = pytest.mark.gpu


def test_order_parameters_of_the_golden_frames(lib):
    import nwgb

    g = dict(np.load(GOLDEN / "order_2d.npz"))
    for name in [str(x) for x in g["names"]]:
        r, L, box = g[f"{name}_r"], int(g[f"{name}_L"]), g[f"{name}_box"]
        cfg = wca_config(len(r) // L, L, (float(box[0]), float(box[1])), lib=lib)
        pos = np.zeros((len(r), 4), np.float32)
        pos[:, :3] = r
        pos[:, 3] = cfg.radius
        with nwgb.System(cfg) as s:
            s.set_array(abi.NW_POSITION, pos)
            got = s.observe()
        want = obs.order_parameters(obs.tangents(r, L))
        assert got["n_tangents"] == want["n_tangents"] == len(r) - 2
        for k in ("s_q3", "s_2d", "polar"):
            assert abs(got[k] - want[k]) < 1e-6, (name, k, got[k], want[k])


@pytest.mark.parametrize("min_image", [False, True])
def test_observables_of_a_simulated_state(lib, min_image):
    import nwgb

    cfg = wca_config(120, 10, (50.0, 50.0), srd=True, seed=3, lib=lib)
    pos, vel = initial_state(cfg, seed=3)
    nb = cfg.n_beads
    box = [cfg.box[a] if cfg.boundary[a] == abi.NW_PERIODIC else 0.0 for a in range(3)]
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.observe_reset()
        unwrapped = pos[:nb, :3].astype(np.float64)
        last = pos[:nb, :3].astype(np.float64)
        for _ in range(6):
            s.step(7, cfg.dt)
            s.sync()
            got = s.observe(min_image=min_image, msd=True)
            p = s.get_array(abi.NW_POSITION)
            v = s.get_array(abi.NW_VELOCITY)
            cur = p[:nb, :3].astype(np.float64)
            d = cur - last
            for a in range(3):
                if box[a] > 0:
                    d[:, a] -= box[a] * np.round(d[:, a] / box[a])
            unwrapped += d
            last = cur
            msd = ((unwrapped - pos[:nb, :3].astype(np.float64)) ** 2).sum(1).mean()
            t = obs.tangents(p[:nb], cfg.filament_size, box if min_image else None)
            want = obs.order_parameters(t)
            for k in ("s_q3", "s_2d", "polar"):
                assert abs(got[k] - want[k]) < 1e-6, (k, got[k], want[k])
            assert abs(got["bead_temperature"] - obs.temperature(v[:nb], cfg.dim)) <= 1e-12 * got["bead_temperature"]
            assert abs(got["solvent_temperature"] - obs.temperature(v[nb:], cfg.dim)) <= \
                1e-12 * got["solvent_temperature"]
            # the oracle's unwrapping adds float64 displacements; the device adds whole boxes
            assert abs(got["msd"] - msd) <= 1e-9 * max(msd, 1e-12), (got["msd"], msd)


def test_velocity_correlation_sums(lib):
    import nwgb

    cfg = wca_config(200, 10, (80.0, 80.0), seed=5, lib=lib)
    pos, vel = initial_state(cfg, seed=5)
    rng = np.random.default_rng(9)
    n = 40000
    i = rng.integers(0, cfg.n_beads, n).astype(np.uint32)
    j = rng.integers(0, cfg.n_beads - 1, n).astype(np.uint32)
    j = j + (j >= i)
    box = [cfg.box[0], cfg.box[1], 0.0]
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.step(20, cfg.dt)
        s.sync()
        p, v = s.get_array(abi.NW_POSITION), s.get_array(abi.NW_VELOCITY)
        sd, sw = s.velocity_correlation(i, j, 8.0, 32)
        sd2, sw2 = s.velocity_correlation(i, j, 8.0, 32)
    wd, ww = obs.velocity_correlation_sums(p, v, i, j, box, 8.0, 32)
    assert np.array_equal(sd, sd2) and np.array_equal(sw, sw2)  # fixed-order sums
    assert np.allclose(sw, ww, rtol=1e-10, atol=1e-12)
    assert np.allclose(sd, wd, rtol=1e-10, atol=1e-12 * np.abs(wd).max())
    assert sw.sum() > 100


@pytest.mark.parametrize("shift", [(0.0, 0.0, 0.0), (0.37, -0.21, 0.0)])
def test_srd_temperature_histogram(lib, shift):
    import nwgb

    cfg = wca_config(80, 10, (40.0, 40.0), srd=True, seed=2, lib=lib)
    pos, vel = initial_state(cfg, seed=2)
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.step(25, cfg.dt)
        s.sync()
        p, v = s.get_array(abi.NW_POSITION), s.get_array(abi.NW_VELOCITY)
        got = s.srd_temperature_histogram(0.5, 50, shift)
    per = [cfg.boundary[a] == abi.NW_PERIODIC for a in range(3)]
    want = obs.srd_temperature_histogram(p, v, list(cfg.srd_grid), list(cfg.srd_cell_size), list(cfg.origin),
                                         list(cfg.box), per, cfg.dim, shift, 0.5, 50)
    assert np.array_equal(got, want), (got, want)
    assert got[-1] > 0.9 * cfg.n_srd_cells
