"""Positions set between updates of a Verlet-list system: the move is added
to the lists' displacement bound instead of forcing a rebuild.  Setting the
positions the system already holds leaves the trajectory bit-identical; a
small move keeps the lists and tracks a rebuilt system to FP32 summation
order; a move beyond half the skin rebuilds, exactly as a fresh list would."""
from __future__ import annotations

import numpy as np
import pytest

from parity import update_err
from nwgb import abi
from nwgb.init import initial_state, wca_config

pytestmark = pytest.mark.gpu


def verlet_system(lib, srd=False):
    import nwgb

    cfg = wca_config(300, 10, (100.0, 100.0), srd=srd, seed=3, lib=lib)
    cfg.strategy = abi.NW_STRATEGY_VERLET
    pos, vel = initial_state(cfg, seed=3)
    s = nwgb.System(cfg)
    s.set_array(abi.NW_POSITION, pos)
    s.set_array(abi.NW_VELOCITY, vel)
    return cfg, s


def state(s):
    return s.get_array(abi.NW_POSITION), s.get_array(abi.NW_VELOCITY)


@pytest.mark.parametrize("srd", [False, True])
def test_setting_unchanged_positions_keeps_the_trajectory(lib, srd):
    cfg, a = verlet_system(lib, srd)
    _, b = verlet_system(lib, srd)
    with a, b:
        a.step(25, cfg.dt)
        b.step(25, cfg.dt)
        nb = cfg.n_beads
        for k in range(30):
            p = b.get_array(abi.NW_POSITION, 0, nb)
            b.set_array(abi.NW_POSITION, p, 0)  # same positions, through the staging path
            a.step(1, cfg.dt)
            b.step(1, cfg.dt)
        a.sync()
        b.sync()
        pa, va = state(a)
        pb, vb = state(b)
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)


def test_small_move_keeps_lists_and_tracks_a_rebuilt_system(lib):
    cfg, a = verlet_system(lib)
    _, b = verlet_system(lib)
    with a, b:
        a.step(20, cfg.dt)
        b.step(20, cfg.dt)
        nb = cfg.n_beads
        rng = np.random.default_rng(1)
        p = a.get_array(abi.NW_POSITION, 0, nb)
        p[:, :2] += rng.uniform(-0.02, 0.02, (nb, 2)).astype(np.float32)
        a.set_array(abi.NW_POSITION, p, 0)                 # staged: bound grows by < 0.03
        b.set_config(b.config)                              # forces a rebuild at the next step
        b.set_array(abi.NW_POSITION, p, 0)
        a.step(20, cfg.dt)
        b.step(20, cfg.dt)
        a.sync()
        b.sync()
        pa, _ = state(a)
        pb, _ = state(b)
    # the same trajectory up to FP32 summation order: per bead, the positions
    # agree to 1e-5 of the displacement since they were set
    assert update_err(pa[:nb], pb[:nb], p, None) < 1e-5


def test_large_move_rebuilds_the_lists(lib):
    """Beads moved by a whole list radius: kept lists would miss the new
    contacts, so the bound must trigger a rebuild; the result then equals a
    system whose lists were rebuilt unconditionally."""
    cfg, a = verlet_system(lib)
    _, b = verlet_system(lib)
    with a, b:
        a.step(10, cfg.dt)
        b.step(10, cfg.dt)
        nb = cfg.n_beads
        p = a.get_array(abi.NW_POSITION, 0, nb)
        p[::2, 0] += np.float32(0.4)  # every other bead along x (beyond half the 0.3 skin)
        a.set_array(abi.NW_POSITION, p, 0)
        b.set_config(b.config)
        b.set_array(abi.NW_POSITION, p, 0)
        a.step(5, cfg.dt)
        b.step(5, cfg.dt)
        a.sync()
        b.sync()
        pa, va = state(a)
        pb, vb = state(b)
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)


def test_tangents_read_through_the_device_pointer_are_current(lib):
    """WCA worms' steps store no tangents; asking for the device array computes
    them, so a caller reading the raw pointer (as the reference's host code does
    with copyArrayFromDevice) sees the tangents of the current positions."""
    import ctypes as C

    cfg, s = verlet_system(lib)
    with s:
        s.step(7, cfg.dt)
        want = s.get_array(abi.NW_TANGENT)
        s.step(5, cfg.dt)
        ptr = s.device_ptr(abi.NW_TANGENT)
        raw = np.zeros((cfg.n_beads, 4), dtype=np.float32)
        lib.copyArrayFromDevice(raw.ctypes.data, C.c_void_p(ptr), None, raw.nbytes)
        now = s.get_array(abi.NW_TANGENT)
    assert np.array_equal(raw, now)
    assert not np.array_equal(now, want)  # the worms moved between the two reads
    assert np.allclose(np.linalg.norm(now[:, :2], axis=1), 1.0, atol=1e-5)
