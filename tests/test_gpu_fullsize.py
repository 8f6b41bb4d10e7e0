"""Full-size workloads on the GPU: one step against the FP32 and FP64
oracles (which finish in seconds on the host cores), per bead and per solvent
particle (tests/parity.py), plus size-independent properties (permutation,
sortedness, cell-bound consistency, momentum balance).

Workloads: 4,000 beads (400 x 10) in a 100 x 100 box; 400,000 beads with
4,000,000 SRD solvent particles in 1000 x 1000 (the step ends with a
collision); 2,000,000 beads in 1400 x 1400."""
from __future__ import annotations

import numpy as np
import pytest

from nwgb import abi
from nwgb.init import baseline_config, initial_state
from parity import SOLVENT_FLOOR, TOL, force_err, fp64_bound, update_err, vec_err

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


def periodic_box(cfg):
    return np.array([cfg.box[a] if cfg.boundary[a] == abi.NW_PERIODIC else 0.0 for a in range(3)])


@pytest.mark.parametrize("k,layout", [(0, "patches"), (1, "patches"), (2, "rows")])
def test_full_size_step_matches_oracle(orc, k, layout):
    cfg = baseline_config(k)
    pos, vel = initial_state(cfg, seed=k, layout=layout)
    g = gpu_one_step(cfg, pos, vel)
    nb = cfg.n_beads
    check_sort_properties(g["hash"], g["sorted_index"], g["cell_start"], g["cell_end"], cfg.n_cells)
    z = np.zeros((nb, 4), np.float32)
    st = dict(pos=pos, vel=vel, force=z, force_old=z, tangent=z)
    o = orc.step(cfg, st, 0, cfg.dt, 32)
    o64 = orc.step(cfg, st, 0, cfg.dt, 64, force_scale=True)
    assert np.array_equal(g["hash"], o["hash"])
    assert np.array_equal(g["sorted_index"], o["sorted_index"])
    assert np.array_equal(g["cell_start"], o["cell_start"])
    check_bead_parity(cfg, g, o, o64, pos)
    if cfg.srd_enabled:
        n = nb + cfg.n_solvent
        si = g["srd_sorted_index"]
        assert np.array_equal(np.sort(si), np.arange(n, dtype=np.uint32))
        # the 4M solvent particles after the collision and streaming of step 0,
        # each against the oracle's (both stored in the collision's cell order)
        box = periodic_box(cfg)
        before = np.asarray(o["pos"][nb:], np.float64)[:, :3] - \
            np.asarray(o["vel"][nb:], np.float64)[:, :3] * (cfg.srd_gap * cfg.dt)
        sv = lambda x, y: vec_err(x["vel"][nb:], y["vel"][nb:], SOLVENT_FLOOR)  # noqa: E731
        sp = lambda x, y: update_err(x["pos"][nb:], y["pos"][nb:], before, box, SOLVENT_FLOOR)  # noqa: E731
        for m in (sv, sp):
            assert m(g, o) < TOL
            assert m(g, o64) < fp64_bound(m(o, o64))


def check_bead_parity(cfg, g, o, o64, pos0):
    """Per bead against the FP32 oracle at 1e-5; against FP64 within the FP32
    oracle's own FP64 error (tests/parity.py)."""
    nb = cfg.n_beads
    box = periodic_box(cfg)
    S = o64["force_scale"]
    for m in (lambda x, y: force_err(x["force"], y["force"], S),
              lambda x, y: vec_err(x["vel"][:nb], y["vel"][:nb]),
              lambda x, y: update_err(x["pos"][:nb], y["pos"][:nb], pos0[:nb], box)):
        assert m(g, o) < TOL, m(g, o)
        assert m(g, o64) < fp64_bound(m(o, o64)), (m(g, o64), m(o, o64))


@pytest.mark.parametrize("k,layout", [(1, "patches"), (2, "rows")])
def test_full_size_update_from_forced_state(orc, k, layout):
    """Step 1 from the FP32 oracle's state after step 0 (non-zero forces): the
    velocity-Verlet update of every bead and the next force pass, per bead
    against the FP32 and FP64 oracles."""
    import nwgb

    cfg = baseline_config(k)
    pos, vel = initial_state(cfg, seed=k, layout=layout)
    nb = cfg.n_beads
    z = np.zeros((nb, 4), np.float32)
    s1 = orc.step(cfg, dict(pos=pos, vel=vel, force=z, force_old=z, tangent=z), 0, cfg.dt, 32)
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, s1["pos"])
        s.set_array(abi.NW_VELOCITY, s1["vel"])
        s.set_array(abi.NW_FORCE, s1["force"])
        s.set_array(abi.NW_FORCE_OLD, s1["force_old"])
        s.set_step(1)
        s.step(1, cfg.dt)
        s.sync()
        g = {k_: s.get_array(a) for k_, a in (("pos", abi.NW_POSITION), ("vel", abi.NW_VELOCITY),
                                             ("force", abi.NW_FORCE), ("force_old", abi.NW_FORCE_OLD),
                                             ("sorted_index", abi.NW_SORTED_INDEX))}
    st = dict(pos=s1["pos"], vel=s1["vel"], force=s1["force"], force_old=s1["force_old"], tangent=s1["tangent"])
    o = orc.step(cfg, st, 1, cfg.dt, 32)
    o64 = orc.step(cfg, st, 1, cfg.dt, 64, force_scale=True)
    assert np.array_equal(g["sorted_index"], o["sorted_index"])
    assert np.array_equal(g["force_old"][:, :3], s1["force"][:, :3])
    check_bead_parity(cfg, g, o, o64, s1["pos"])
    if cfg.srd_enabled:  # no collision in step 1: the solvent is left as it was
        assert np.array_equal(g["pos"][nb:], s1["pos"][nb:])
        assert np.array_equal(g["vel"][nb:], s1["vel"][nb:])


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
