"""Known-answer and property tests of the CPU oracle (derived from the force
laws and from the Philox publication; no GPU)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from nwgb import abi
from nwgb.init import initial_state, wca_config


def test_philox_known_answers(orc):
    # Random123 known-answer vectors for Philox4x32-10
    assert orc.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert orc.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_normals_are_standard(orc):
    z = np.array([orc.normal4(5, i, 3, 1) for i in range(20000)]).ravel()
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1.0) < 0.02
    u = np.array([orc.uniform4(5, i, 3, 2) for i in range(5000)]).ravel()
    assert u.min() > 0.0 and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.01


def two_bead_cfg(lib, model, L=1):
    c = abi.default_config(model, 2 // L if L else 2, L, (16, 16, 1), False, lib)
    return c


def test_wca_two_bead_force(lib, orc):
    cfg = wca_config(2, 1, (20.0, 20.0), lib=lib)
    for r in (0.95, 1.0, 1.05, 1.12):
        pos = np.zeros((2, 4), np.float32)
        pos[1, 0] = r
        f = orc.pair_wca_bruteforce(cfg, np.zeros((2, 4)), pos, 64)
        rr = float(np.float32(r)) ** 2
        expect = 24.0 * (2.0 / rr ** 7 - 1.0 / rr ** 4) * float(np.float32(r))  # F_0 = f(rr) * (r_0 - r_1)
        assert f[0, 0] == pytest.approx(-expect, rel=1e-12)
        assert f[1, 0] == pytest.approx(expect, rel=1e-12)
    pos = np.zeros((2, 4), np.float32)
    pos[1, 0] = 1.13  # beyond 2^(1/6)
    assert np.all(orc.pair_wca_bruteforce(cfg, np.zeros((2, 4)), pos, 64) == 0.0)


def test_wca_bond_and_drive(lib, orc):
    cfg = wca_config(1, 2, (20.0, 20.0), lib=lib)
    cfg.bend_k = 0.0
    for r in (0.7, 0.8, 0.9):
        pos = np.zeros((2, 4), np.float32)
        pos[1, 0] = r
        f, _ = orc.filament(cfg, np.zeros((2, 4)), np.zeros((2, 4)), pos, 64)
        rr = float(np.float32(r))
        # harmonic bond pulls toward r0, drive F_act along +x on bead 0 only
        r0 = float(np.float32(0.8))
        assert f[0, 0] == pytest.approx(57.0 * (rr - r0) + 0.5, abs=1e-9)
        assert f[1, 0] == pytest.approx(-57.0 * (rr - r0), abs=1e-9)


def test_bending_right_angle_and_straight(lib, orc):
    cfg = abi.default_config(abi.NW_MODEL_REF_DEM, 1, 3, (16, 16, 1), False, lib)
    cfg.bend_k = 2.0
    pos = np.zeros((3, 4), np.float32)
    pos[1] = (1.0, 0.0, 0.0, 0.5)
    pos[2] = (1.0, 1.0, 0.0, 0.5)  # 90 degree bend
    f, t = orc.filament(cfg, np.zeros((3, 4)), np.zeros((3, 4)), pos, 64)
    # U = k (1 - cos theta): F_0 = -k (r_jk - r_ij cos) / (|r_ij||r_jk|) = -k (0, 1, 0)
    assert np.allclose(f[0, :3], [0.0, -2.0, 0.0]) and np.allclose(f[2, :3], [2.0, 0.0, 0.0])
    assert np.allclose(f.sum(0)[:3], 0.0)
    assert np.allclose(t[0, :3], [1, 0, 0]) and np.allclose(t[1, :3], [1 / math.sqrt(2), 1 / math.sqrt(2), 0])
    pos[2] = (2.0, 0.0, 0.0, 0.5)  # straight: no force
    f, _ = orc.filament(cfg, np.zeros((3, 4)), np.zeros((3, 4)), pos, 64)
    assert np.allclose(f[:, :3], 0.0)


def test_hash_cell_boundaries(lib, orc):
    cfg = abi.default_config(abi.NW_MODEL_REF_DEM, 1, 1, (8, 8, 1), False, lib)
    # origin -4, cell 1: exact cell edges map to the upper cell; -4 -> 0; 4 -> 8 & 7 = 0 (mask wrap).
    # 3.9999995 + 4 = 8 - 2^-21 stays below 8 (cell 7); 3.9999998 + 4 rounds to 8.0 in FP32 (cell 0).
    pts = np.array([[-4.0, -4.0, 0.0, 0.5], [-3.0, -4.0, 0.0, 0.5], [3.9999995, 3.9999995, 0, 0.5],
                    [4.0, 0.0, 0.0, 0.5], [-4.0000005, 0.0, 0.0, 0.5], [3.9999998, 0.0, 0.0, 0.5]], np.float32)
    h, _ = orc.calc_hash(cfg, pts)
    assert list(h) == [0, 1, 63, 4 * 8 + 0, 4 * 8 + 7, 4 * 8 + 0]
    # modulo wrap for a non-power-of-two grid
    c2 = wca_config(1, 1, (10.0 * 1.12246205, 10.0 * 1.12246205), lib=lib)
    p2 = np.array([[c2.origin[0] - 0.5 * c2.cell_size[0], c2.origin[1] + 0.1, 0, 0.5]], np.float32)
    h2, _ = orc.calc_hash(c2, p2)
    assert h2[0] == 9  # x wraps to the last column, y in row 0


def test_srd_rotation_of_known_vector(lib, orc):
    cfg = abi.default_config(abi.NW_MODEL_WCA_WORMS, 0, 1, (4, 4, 1), True, lib)
    cfg.srd_thermostat = abi.NW_SRD_THERMO_NONE
    cfg.num_solvent = 2
    pos = np.array([[-1.9, -1.9, 0, 0], [-1.8, -1.8, 0, 0]], np.float32)
    vel = np.array([[1.0, 0.0, 0.0, 1.0], [-1.0, 0.0, 0.0, 1.0]], np.float32)
    for u, sgn in ((0.9, 1.0), (0.1, -1.0)):
        rot = np.full(cfg.n_srd_cells, u, np.float32)
        out = orc.srd(cfg, pos, vel, 0, 2, [0, 0, 0], rot, 0, 0.0, 64)
        a = sgn * cfg.srd_alpha
        assert np.allclose(out["vel"][0, :2], [math.cos(a), math.sin(a)], atol=1e-6)
        assert np.allclose(out["vel"][1, :2], [-math.cos(a), -math.sin(a)], atol=1e-6)


def test_pair_forces_obey_newtons_third_law(lib, orc):
    cfg = wca_config(30, 10, (30.0, 30.0), seed=2, lib=lib)
    pos, vel = initial_state(cfg, seed=2)
    pos[:, :2] += np.random.default_rng(0).normal(0, 0.05, (cfg.n_beads, 2)).astype(np.float32)
    b = orc.bead_sort(cfg, pos)
    z = np.zeros_like(pos)
    f = orc.pair(cfg, z, pos, vel, z, b["sorted_index"], b["cell_start"], b["cell_end"], 64)
    assert np.abs(f[:, :3].sum(0)).max() < 1e-9 * np.abs(f).max() * cfg.n_beads


def test_wca_forces_are_permutation_equivariant(lib, orc):
    """Relabelling filaments permutes the forces and nothing else."""
    cfg = wca_config(30, 10, (30.0, 30.0), seed=4, lib=lib)
    pos, vel = initial_state(cfg, seed=4)
    L = cfg.filament_size
    perm_f = np.random.default_rng(1).permutation(cfg.num_filaments)
    perm = (perm_f[:, None] * L + np.arange(L)[None, :]).ravel()
    z = np.zeros_like(pos)

    def forces(p):
        f, t = orc.filament(cfg, z, z, p, 64)
        b = orc.bead_sort(cfg, p)
        return orc.pair(cfg, f, p, z, t, b["sorted_index"], b["cell_start"], b["cell_end"], 64)

    f0 = forces(pos)
    f1 = forces(pos[perm])
    assert np.allclose(f1, f0[perm], rtol=1e-12, atol=1e-12)


def test_srd_conserves_momentum_and_energy_without_thermostat(lib, orc):
    cfg = wca_config(50, 10, (40.0, 40.0), srd=True, seed=5, lib=lib)
    cfg.srd_thermostat = abi.NW_SRD_THERMO_NONE
    pos, vel = initial_state(cfg, seed=5)
    n = cfg.n_beads + cfg.n_solvent
    out = orc.srd(cfg, pos, vel, cfg.n_beads, cfg.n_solvent, orc.srd_shift(cfg, 0), None, 0, 0.0, 64)
    m = vel[:, 3:4].astype(np.float64)
    p0 = (m * vel[:, :3]).sum(0)
    p1 = (m * out["vel"][:, :3]).sum(0)
    e0 = 0.5 * (m * vel[:, :3] ** 2).sum()
    e1 = 0.5 * (m * out["vel"][:, :3] ** 2).sum()
    assert np.abs(p1 - p0).max() < 1e-9 * n
    assert abs(e1 - e0) < 1e-9 * e0


def test_srd_cell_thermostat_hits_target(lib, orc):
    cfg = wca_config(10, 10, (30.0, 30.0), srd=True, seed=6, lib=lib)
    pos, vel = initial_state(cfg, seed=6)
    vel[:, :2] *= 3.0  # hot start
    out = orc.srd(cfg, pos, vel, cfg.n_beads, cfg.n_solvent, orc.srd_shift(cfg, 0), None, 0, 0.0, 64)
    si, cs, ce, cm = out["sorted_index"], out["cell_start"], out["cell_end"], out["cell_mean"]
    v = out["vel"].astype(np.float64)
    for c in np.flatnonzero(cs != 0xFFFFFFFF)[:200]:
        members = si[cs[c]:ce[c]]
        if len(members) < 2:
            continue
        rel = v[members, :2] - cm[c, :2]
        ke = 0.5 * (rel ** 2).sum()
        assert ke == pytest.approx((len(members) - 1) * cfg.srd_kT, rel=1e-9)
