"""Pin the CPU oracle to the reference: every oracle routine reproduces the
golden vectors that the reference's own kernels produced (tests/golden,
generated by tests/golden/make_golden.py)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, rel_err
from nwgb.abi import NwConfig


def load(name):
    d = dict(np.load(GOLDEN / name))
    cfg = NwConfig.from_buffer_copy(d["cfg"].tobytes())
    return cfg, d


REF_CASES = ["ref_dem_2d.npz", "ref_dem_3d_walls.npz"]


@pytest.mark.parametrize("name", REF_CASES)
def test_integrate_matches_reference(orc, name):
    cfg, d = load(name)
    p, v, f, fo = orc.integrate(cfg, d["pos_in"], d["vel_in"], d["force_in"], d["force_old_in"], float(d["dt"]), 32)
    assert np.array_equal(p, d["int_pos"])
    assert np.array_equal(v, d["int_vel"])
    assert np.array_equal(f, d["int_force"])
    assert np.array_equal(fo, d["int_force_old"])


@pytest.mark.parametrize("name", REF_CASES)
def test_reverse_matches_reference(orc, name):
    cfg, d = load(name)
    c2 = cfg.copy()
    c2.reverse_probability = 0.3
    f, fo, v, p = orc.reverse(c2, d["int_force"], d["int_force_old"], d["int_vel"], d["int_pos"], d["uniform"], 32)
    assert np.array_equal(p, d["rev_pos"]) and np.array_equal(v, d["rev_vel"])
    assert np.array_equal(f, d["rev_force"]) and np.array_equal(fo, d["rev_force_old"])


@pytest.mark.parametrize("name", REF_CASES)
def test_langevin_and_bending_match_reference(orc, name):
    cfg, d = load(name)
    lf = orc.langevin(cfg, d["int_force"], d["int_vel"], d["noise"], 32)
    assert np.array_equal(lf, d["lang_force"])
    ff, tt = orc.filament(cfg, lf, d["tan_in"], d["int_pos"], 32)
    assert np.array_equal(ff, d["fil_force"])
    assert np.array_equal(tt, d["fil_tan"])
    ff64, tt64 = orc.filament(cfg, lf, d["tan_in"], d["int_pos"], 64)
    assert rel_err(ff64, d["fil_force"]) < 1e-5


@pytest.mark.parametrize("name", REF_CASES)
def test_hash_sort_cells_match_reference(orc, name):
    cfg, d = load(name)
    h, idx = orc.calc_hash(cfg, d["int_pos"])
    assert np.array_equal(h, d["hash"])
    sh, si = orc.sort_by_key(h, idx)
    assert np.array_equal(sh, d["sorted_hash"]) and np.array_equal(si, d["sorted_index"])
    cs, ce = orc.cell_bounds(sh, cfg.n_cells)
    assert np.array_equal(cs, d["cell_start"])
    ne = cs != 0xFFFFFFFF
    assert np.array_equal(ce[ne], d["cell_end"][ne])


@pytest.mark.parametrize("name", REF_CASES)
def test_pair_ref_dem_matches_reference(orc, name):
    cfg, d = load(name)
    f = orc.pair(cfg, d["fil_force"], d["int_pos"], d["int_vel"], d["fil_tan"], d["sorted_index"], d["cell_start"],
                 d["cell_end"], 32)
    assert np.array_equal(f, d["collide_force"])
    f64 = orc.pair(cfg, d["fil_force"], d["int_pos"], d["int_vel"], d["fil_tan"], d["sorted_index"],
                   d["cell_start"], d["cell_end"], 64)
    assert rel_err(f64, d["collide_force"]) < 1e-5


def test_srd_matches_reference(orc):
    cfg, d = load("ref_srd_2d.npz")
    h, _ = orc.calc_hash_srd(cfg, d["pos_in"], d["shift"])
    assert np.array_equal(h, d["hash"])
    out = orc.srd(cfg, d["pos_in"], d["vel_in"], cfg.n_beads, cfg.n_solvent, d["shift"], d["uniform"], 0,
                  float(d["dt_srd"]), 32)
    assert np.array_equal(out["sorted_index"], d["sorted_index"])
    assert np.array_equal(out["cell_start"], d["cell_start"])
    ne = out["cell_start"] != 0xFFFFFFFF
    assert np.array_equal(out["cell_end"][ne], d["cell_end"][ne])
    # the rotation uses sinf/cosf of the C library: equal to rounding
    assert np.abs(out["cell_mean"] - d["com"]).max() <= 1e-6 * max(1.0, np.abs(d["com"]).max())
    assert np.abs(out["vel"] - d["vel_out"]).max() <= 2e-6 * np.abs(d["vel_out"]).max()
    assert np.abs(out["pos"] - d["pos_out"]).max() <= 2e-6 * np.abs(d["pos_out"]).max()


def test_wca_forces_match_archived_kernels(orc):
    cfg, d = load("wca_archived_2d.npz")
    z = np.zeros_like(d["pos"])
    for prec in (32, 64):
        f, t = orc.filament(cfg, z, z, d["pos"], prec)
        b = orc.bead_sort(cfg, d["pos"])
        f = orc.pair(cfg, f, d["pos"], z, t, b["sorted_index"], b["cell_start"], b["cell_end"], prec)
        # summation order differs from the archived kernels: FP32 rounding only
        assert rel_err(f, d["force_conservative"]) < 1e-5
    # noise + drag path of InterForceKernel: Langevin with the injected draws
    noise = d["noise"].astype(np.float64) * float(d["noise_scale"])
    noise[:, 2:] = 0.0
    f, t = orc.filament(cfg, orc.langevin(cfg, z, d["vel"], noise, 64), z, d["pos"], 64)
    b = orc.bead_sort(cfg, d["pos"])
    f = orc.pair(cfg, f, d["pos"], d["vel"], t, b["sorted_index"], b["cell_start"], b["cell_end"], 64)
    assert rel_err(f, d["force_total"]) < 1e-5


def test_wca_constants_match_archived_derivation(orc):
    _, d = load("wca_archived_2d.npz")
    s6, two_s6, amp, rmin, r2min, rcut, r2cut = d["lj_constants"]
    assert (s6, two_s6, amp) == (1.0, 2.0, 24.0)
    assert rcut == np.float32(1.12246205) and r2cut == np.float32(1.12246205) * np.float32(1.12246205)
