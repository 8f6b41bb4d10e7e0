"""Initial states and the workload configurations.

``baseline_config(k)`` builds the five workloads the engine is measured on
(2D WCA worms; the SRD and large dense systems; batched and adjoint forms
reuse the small one).  Initial states are seeded and reproducible:
straight worms with bond spacing r0 on a jittered lattice of randomly
turned patches (or by random sequential addition for dilute systems, or in
aligned rows for the dense nematic start), Maxwell-Boltzmann velocities, SRD
solvent uniform in the box.  ``reference_reset`` restates the reference's own
ParticleSystem::reset lattice (simulation/particleSystem.cpp:583-678),
drawing from the C library's rand() exactly as the reference does.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import abi
from .abi import NwConfig


def wca_config(num_filaments: int, filament_size: int, box=(100.0, 100.0), *, srd: bool = False,
               srd_density: float = 4.0, activity: float = 0.5, bend_k: float = 10.0, seed: int = 0,
               lib=None) -> NwConfig:
    """2D WCA worm configuration in a periodic box (cells of edge >= 2^(1/6) sigma)."""
    lib = lib or abi.load_library()
    rc = 1.12246205
    gx = max(1, int(math.floor(box[0] / rc)))
    gy = max(1, int(math.floor(box[1] / rc)))
    c = abi.default_config(abi.NW_MODEL_WCA_WORMS, num_filaments, filament_size, (gx, gy, 1), False, lib)
    c.cell_size[0] = box[0] / gx
    c.cell_size[1] = box[1] / gy
    abi.check(lib.nw_config_finalize(C.byref(c)))
    c.activity = activity
    c.bend_k = bend_k
    c.seed = seed
    if srd:
        c.srd_enabled = 1
        c.srd_grid[0] = max(1, int(round(box[0])))
        c.srd_grid[1] = max(1, int(round(box[1])))
        c.srd_grid[2] = 1
        c.srd_cell_size[0] = c.box[0] / c.srd_grid[0]
        c.srd_cell_size[1] = c.box[1] / c.srd_grid[1]
        c.srd_cell_size[2] = c.box[2]
        c.num_solvent = int(round(srd_density * c.srd_grid[0] * c.srd_grid[1]))
        c.srd_alpha = math.radians(130.0)
        c.srd_gap = 10
        c.srd_kT = c.kT
        c.srd_shift_lo = -0.5
        c.srd_rotate_beads = 1
        c.srd_thermostat = abi.NW_SRD_THERMO_CELL_REL
    return c


def baseline_config(k: int, lib=None, seed: int = 0) -> NwConfig:
    """Workload k: 0 small 2D (400x10, box 100); 1 SRD (20000x20, box 1000,
    4M solvent); 2 large dense (100000x20, box 1400, F_act = 1)."""
    if k == 0:
        return wca_config(400, 10, (100.0, 100.0), seed=seed, lib=lib)
    if k == 1:
        return wca_config(20000, 20, (1000.0, 1000.0), srd=True, seed=seed, lib=lib)
    if k == 2:
        return wca_config(100000, 20, (1400.0, 1400.0), activity=1.0, seed=seed, lib=lib)
    raise ValueError(k)


def batch_configs(n_replicas: int = 256, seed: int = 0, lib=None, worms=(50, 2000), beads=(5, 30),
                  activity=(0.0, 2.0), bend_k=(1.0, 20.0), packing=(0.3, 0.6)) -> list:
    """Replicas of uneven size for the batched engine: per replica worm count
    and length uniform in the given integer ranges, F_act, k_bend and packing
    fraction uniform in theirs, box side sqrt(N pi/4 / packing) for N beads of
    unit diameter, seed = seed + r."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n_replicas):
        M = int(rng.integers(worms[0], worms[1] + 1))
        L = int(rng.integers(beads[0], beads[1] + 1))
        phi = float(rng.uniform(*packing))
        side = math.sqrt(M * L * math.pi / 4.0 / phi)
        c = wca_config(M, L, (side, side), activity=float(rng.uniform(*activity)),
                       bend_k=float(rng.uniform(*bend_k)), seed=seed + r, lib=lib)
        out.append(c)
    return out


def _worm_beads(head, angle, L, spacing):
    d = np.array([math.cos(angle), math.sin(angle)])
    return head[None, :] + np.arange(L)[:, None] * spacing * d[None, :]


def rsa_worms(cfg: NwConfig, rng: np.random.Generator, *, min_sep: float = 0.9, angle_fn=None,
              max_attempts: int = 200) -> np.ndarray:
    """Random sequential addition of straight worms (bond spacing r0) in the
    periodic box; returns bead positions (n, 2) in storage order."""
    M, L = int(cfg.num_filaments), int(cfg.filament_size)
    box = np.array([cfg.box[0], cfg.box[1]], dtype=np.float64)
    org = np.array([cfg.origin[0], cfg.origin[1]], dtype=np.float64)
    spacing = float(cfg.bond_r0)
    cell = max(min_sep, 1e-3)
    G = np.maximum(1, np.floor(box / cell).astype(int))
    csz = box / G
    grid: dict = {}
    out = np.zeros((M * L, 2))
    ms2 = min_sep * min_sep
    for w in range(M):
        for _ in range(max_attempts):
            head = org + rng.random(2) * box
            ang = angle_fn(rng) if angle_fn else rng.random() * 2.0 * math.pi
            beads = _worm_beads(head, ang, L, spacing)
            beads = org + np.mod(beads - org, box)
            ci = np.floor((beads - org) / csz).astype(int) % G
            ok = True
            for b in range(L):
                cx, cy = ci[b]
                for dx in (-1, 0, 1):
                    for dy in (-1, 0, 1):
                        lst = grid.get(((cx + dx) % G[0], (cy + dy) % G[1]))
                        if not lst:
                            continue
                        other = np.asarray(lst)
                        d = other - beads[b]
                        d -= box * np.round(d / box)
                        if np.any((d * d).sum(1) < ms2):
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                break
        else:
            raise RuntimeError(f"could not place worm {w} after {max_attempts} attempts")
        out[w * L:(w + 1) * L] = beads
        for b in range(L):
            grid.setdefault((ci[b][0], ci[b][1]), []).append(beads[b])
    return out


def lattice_patches(cfg: NwConfig, rng: np.random.Generator, pitch: float = 1.13) -> np.ndarray:
    """Straight worms on a jittered square lattice of sites, each site a patch of
    k parallel worms (row pitch just beyond the WCA cut-off) turned to a
    uniformly random angle, with random polarity per worm.  Patches never
    overlap: the lattice spacing exceeds each patch's bounding circle.  k is
    the smallest patch size whose sites hold all worms; sites are filled in
    random order."""
    M, L = int(cfg.num_filaments), int(cfg.filament_size)
    if M == 0:
        return np.zeros((0, 2))
    box = np.array([cfg.box[0], cfg.box[1]], dtype=np.float64)
    org = np.array([cfg.origin[0], cfg.origin[1]], dtype=np.float64)
    spacing = float(cfg.bond_r0)
    length = (L - 1) * spacing + 1.0
    for k in range(1, 64):
        rho = math.hypot(length / 2.0, k * pitch / 2.0)
        nx = int(box[0] // (2.0 * rho + 0.05))
        ny = int(box[1] // (2.0 * rho + 0.05))
        if nx * ny * k >= M:
            break
    else:
        raise RuntimeError("box too small for the worms")
    sx, sy = box[0] / nx, box[1] / ny
    slack = np.array([sx, sy]) - 2.0 * rho
    sites = rng.permutation(nx * ny)[: int(math.ceil(M / k))]
    out = np.zeros((M * L, 2))
    w = 0
    for s in sites:
        ix, iy = divmod(int(s), ny)
        centre = org + np.array([(ix + 0.5) * sx, (iy + 0.5) * sy]) + (rng.random(2) - 0.5) * slack
        ang = rng.random() * 2.0 * math.pi
        d = np.array([math.cos(ang), math.sin(ang)])
        nrm = np.array([-d[1], d[0]])
        for r in range(k):
            if w >= M:
                break
            off = (r - (k - 1) / 2.0) * pitch
            sign = 1.0 if rng.random() < 0.5 else -1.0
            beads = centre[None, :] + off * nrm[None, :] + sign * (np.arange(L) - (L - 1) / 2.0)[:, None] * spacing * d
            out[w * L:(w + 1) * L] = org + np.mod(beads - org, box)
            w += 1
    return out


def aligned_rows(cfg: NwConfig, rng: np.random.Generator, spread_deg: float = 10.0) -> np.ndarray:
    """Worms along x in rows (dense nematic start): rows of pitch box_y / n_rows,
    random polarity and row offset; the angular spread is limited to what the
    row pitch allows without overlap."""
    M, L = int(cfg.num_filaments), int(cfg.filament_size)
    box = np.array([cfg.box[0], cfg.box[1]])
    org = np.array([cfg.origin[0], cfg.origin[1]])
    spacing = float(cfg.bond_r0)
    length = (L - 1) * spacing
    per_row = int(box[0] // (length + 1.0))
    rows = int(math.ceil(M / per_row))
    pitch = box[1] / rows
    if pitch < 1.0:
        raise RuntimeError("box too small for aligned rows")
    max_ang = math.atan2(max(pitch - 1.0, 0.0), length) * 0.9
    out = np.zeros((M * L, 2))
    slot_w = box[0] / per_row
    for w in range(M):
        r, s = divmod(w, per_row)
        ang = float(np.clip(rng.normal(0.0, math.radians(spread_deg)), -max_ang, max_ang))
        if rng.random() < 0.5:
            ang += math.pi
        centre = org + np.array([(s + 0.5) * slot_w + (r % 2) * 0.5 * slot_w, (r + 0.5) * pitch])
        d = np.array([math.cos(ang), math.sin(ang)])
        beads = centre[None, :] + (np.arange(L) - (L - 1) / 2.0)[:, None] * spacing * d[None, :]
        out[w * L:(w + 1) * L] = org + np.mod(beads - org, box)
    return out


def maxwell_boltzmann(n: int, kT: float, mass: float, rng: np.random.Generator, dim: int = 2) -> np.ndarray:
    v = np.zeros((n, 3))
    v[:, :dim] = rng.normal(0.0, math.sqrt(kT / mass), size=(n, dim))
    if n > 1:
        v[:, :dim] -= v[:, :dim].mean(axis=0)
    return v


def initial_state(cfg: NwConfig, seed: int = 0, layout: str = "patches"):
    """Positions and velocities (float32, (n_total, 4)) for a configuration."""
    rng = np.random.default_rng(seed)
    nb = cfg.n_beads
    ns = cfg.n_solvent
    pos = np.zeros((nb + ns, 4), dtype=np.float32)
    vel = np.zeros((nb + ns, 4), dtype=np.float32)
    if layout == "rows":
        xy = aligned_rows(cfg, rng)
    elif layout == "rsa":
        xy = rsa_worms(cfg, rng)
    else:
        xy = lattice_patches(cfg, rng)
    pos[:nb, 0:2] = xy
    pos[:nb, 3] = cfg.radius
    vel[:nb, 0:3] = maxwell_boltzmann(nb, cfg.kT, cfg.mass, rng, cfg.dim)
    vel[:nb, 3] = cfg.mass
    if ns:
        lo = np.array([cfg.origin[0], cfg.origin[1]])
        hi = lo + np.array([cfg.box[0], cfg.box[1]])
        pos[nb:, 0:2] = rng.uniform(lo, hi, size=(ns, 2))
        vel[nb:, 0:3] = maxwell_boltzmann(ns, cfg.srd_kT, cfg.solvent_mass, rng, cfg.dim)
        vel[nb:, 3] = cfg.solvent_mass
    return pos, vel


def reference_reset(cfg: NwConfig, lib=None):
    """The reference's reset() (simulation/particleSystem.cpp:583-678):
    filaments on a lattice along x with spacing bondSpringL, half of them
    flipped, velocities 0.1 * U(-1, 1), solvent uniform with speed scale 5,
    all drawn from the C library's rand() after srand(1) (nw_reference_reset
    in libnwgb).  Returns (pos, vel, tan) as float32 arrays."""
    lib = lib or abi.load_library()
    nb, ns = cfg.n_beads, cfg.n_solvent
    pos = np.zeros((nb + ns, 4), dtype=np.float32)
    vel = np.zeros((nb + ns, 4), dtype=np.float32)
    tan = np.zeros((max(nb, 1), 4), dtype=np.float32)
    abi.check(lib.nw_reference_reset(C.byref(cfg), pos.ctypes.data, vel.ctypes.data, tan.ctypes.data),
              "nw_reference_reset")
    return pos, vel, tan[:nb]
