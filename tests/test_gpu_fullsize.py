"""Full-size workloads on the GPU: one step against the FP32 oracle (which
finishes in seconds on the host cores) plus size-independent properties
(permutation, sortedness, cell-bound consistency, momentum balance)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err
from nwgb import abi
from nwgb.init import baseline_config, initial_state

pytestmark = pytest.mark.gpu


def gpu_one_step(cfg, pos, vel):
    import nwgb

    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.step(1, cfg.dt)
        s.sync()
        out = {k: s.get_array(a) for k, a in (("pos", abi.NW_POSITION), ("vel", abi.NW_VELOCITY),
                                               ("force", abi.NW_FORCE), ("hash", abi.NW_HASH),
                                               ("sorted_index", abi.NW_SORTED_INDEX),
                                               ("cell_start", abi.NW_CELL_START), ("cell_end", abi.NW_CELL_END))}
        if cfg.srd_enabled:
            out["srd_sorted_index"] = s.get_array(abi.NW_SRD_SORTED_INDEX)
            out["srd_cell_start"] = s.get_array(abi.NW_SRD_CELL_START)
            out["srd_cell_end"] = s.get_array(abi.NW_SRD_CELL_END)
    return out


def check_sort_properties(h, si, cs, ce, ncells):
    n = h.shape[0]
    assert np.array_equal(np.sort(si), np.arange(n, dtype=np.uint32))  # a permutation
    sh = h[si]
    assert np.all(np.diff(sh.astype(np.int64)) >= 0)  # sorted by hash
    same = np.diff(sh.astype(np.int64)) == 0
    assert np.all(np.diff(si.astype(np.int64))[same] > 0)  # stable: ties in index order
    counts = np.bincount(sh, minlength=ncells)
    nz = counts > 0
    assert np.all(cs[~nz] == abi.EMPTY)
    assert np.array_equal(ce[nz] - cs[nz], counts[nz])
    assert np.array_equal(sh[cs[nz]], np.flatnonzero(nz))


@pytest.mark.parametrize("k,layout", [(1, "patches"), (2, "rows")])
def test_full_size_step_matches_oracle(orc, k, layout):
    cfg = baseline_config(k)
    pos, vel = initial_state(cfg, seed=k, layout=layout)
    g = gpu_one_step(cfg, pos, vel)
    nb = cfg.n_beads
    check_sort_properties(g["hash"], g["sorted_index"], g["cell_start"], g["cell_end"], cfg.n_cells)
    z = np.zeros((nb, 4), np.float32)
    o = orc.step(cfg, dict(pos=pos, vel=vel, force=z, force_old=z, tangent=z), 0, cfg.dt, 32)
    assert np.array_equal(g["hash"], o["hash"])
    assert np.array_equal(g["sorted_index"], o["sorted_index"])
    assert np.array_equal(g["cell_start"], o["cell_start"])
    for key in ("pos", "vel"):
        assert rel_err(g[key], o[key]) < 1e-5, key
    assert rel_err(g["force"], o["force"]) < 1e-5
    if cfg.srd_enabled:
        n = nb + cfg.n_solvent
        si = g["srd_sorted_index"]
        assert np.array_equal(np.sort(si), np.arange(n, dtype=np.uint32))


def test_full_size_srd_conserves_momentum():
    """WCA SRD collision (beads rotated, relative-velocity thermostat)
    conserves the total momentum of beads + solvent."""
    import nwgb

    cfg = baseline_config(1)
    pos, vel = initial_state(cfg, seed=3)
    n = cfg.n_beads + cfg.n_solvent
    m = vel[:, 3:4].astype(np.float64)
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        p0 = (m * vel[:, :3]).sum(0)
        s.srd_collide(cfg.dt * cfg.srd_gap, (0.3, -0.2, 0.0))
        v1 = s.get_array(abi.NW_VELOCITY)  # solvent now in cell order: masses travel in w
        p1 = (v1[:, 3:4].astype(np.float64) * v1[:, :3]).sum(0)
        # per-particle FP32 rounding (~1e-8 of a velocity ~0.3) summed over 4.4M particles
        assert np.abs(p1 - p0).max() < 1e-3
        si = s.get_array(abi.NW_SRD_SORTED_INDEX)
        assert np.array_equal(np.sort(si), np.arange(n, dtype=np.uint32))


def test_full_size_conservative_forces_sum_to_zero():
    """With drive, drag and noise off, bonded + pair forces balance
    (Newton's third law) over 2M beads."""
    import nwgb

    cfg = baseline_config(2)
    cfg.activity = 0.0
    cfg.gamma = 0.0
    cfg.kT = 0.0
    pos, vel = initial_state(cfg, seed=5, layout="rows")
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, np.zeros_like(vel))
        s.step(1, cfg.dt)
        s.sync()
        f = s.get_array(abi.NW_FORCE).astype(np.float64)
    scale = np.abs(f).sum()
    assert np.abs(f[:, :3].sum(0)).max() < 1e-6 * scale
