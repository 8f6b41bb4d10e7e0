"""Generate the golden vectors in tests/golden/ from the reference's own kernels.

The reference ships no tests or fixtures, so the vectors are produced by
running the reference's kernel source (simulation/particles_kernel_impl.cuh
and the archived worm-force kernels), compiled for the CPU by
oracle/ref_emu, on seeded inputs.  Requires the reference tree at build time
(oracle/_ref/*.so); the committed .npz files are what the tests read.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "nematic-worms_gb300"))
sys.path.insert(0, str(REPO / "oracle"))

import oracle as orc  # noqa: E402
from nwgb import abi  # noqa: E402
from nwgb.init import initial_state, reference_reset, wca_config  # noqa: E402


def cfg_bytes(cfg):
    return np.frombuffer(bytes(cfg), dtype=np.uint8).copy()


def ptr(a):
    return None if a is None else a.ctypes.data


def ref_dem_case(seed: int, grid, nf: int, L: int, boundaries=(0, 0, 0)):
    """One REF_DEM bead pass through the reference kernels."""
    R = orc.ref_modern()
    cfg = abi.default_config(abi.NW_MODEL_REF_DEM, nf, L, grid, False)
    cfg.bond_r0 = 0.8
    cfg.bend_k = 10.0
    cfg.activity = 0.5
    cfg.gamma = 2.0
    cfg.kT = 0.1
    cfg.spring = 57.0
    cfg.boundary[0], cfg.boundary[1], cfg.boundary[2] = boundaries
    pos, vel, tan = reference_reset(cfg)
    rng = np.random.default_rng(seed)
    nb = cfg.n_beads
    pos[:nb, :2] += rng.normal(0.0, 0.08, (nb, 2)).astype(np.float32)
    vel[:nb, :3] += rng.normal(0.0, 0.3, (nb, 3)).astype(np.float32)
    force = rng.normal(0.0, 1.0, (nb, 4)).astype(np.float32)
    force[:, 3] = 0.0
    force_old = rng.normal(0.0, 1.0, (nb, 4)).astype(np.float32)
    force_old[:, 3] = 0.0
    noise = rng.normal(0.0, 0.6, (nb, 4)).astype(np.float32)
    uniform = rng.random(nf).astype(np.float32)
    dt = np.float32(0.005)
    out = dict(cfg=cfg_bytes(cfg), pos_in=pos.copy(), vel_in=vel.copy(), tan_in=tan.copy(), force_in=force.copy(),
               force_old_in=force_old.copy(), noise=noise, uniform=uniform, dt=dt)
    # integrate
    p, v, f, fo = pos.copy(), vel.copy(), force.copy(), force_old.copy()
    R.ref_integrate(C.byref(cfg), ptr(p), ptr(v), ptr(f), ptr(fo), float(dt), nb)
    out.update(int_pos=p.copy(), int_vel=v.copy(), int_force=f.copy(), int_force_old=fo.copy())
    # reverse (probability 0.3 on the injected uniforms)
    c2 = cfg.copy()
    c2.reverse_probability = 0.3
    rf, rfo, rv, rp = f.copy(), fo.copy(), v.copy(), p.copy()
    R.ref_reverse(C.byref(c2), ptr(rf), ptr(rfo), ptr(rv), ptr(rp), ptr(uniform), nf)
    out.update(rev_pos=rp, rev_vel=rv, rev_force=rf, rev_force_old=rfo)
    # Langevin with the injected noise
    lf = f.copy()
    R.ref_langevin(C.byref(cfg), ptr(lf), ptr(v), ptr(noise), nb)
    out.update(lang_force=lf.copy())
    # bending + tangents
    ff, tt = lf.copy(), tan.copy()
    R.ref_filament_forces(C.byref(cfg), ptr(ff), ptr(tt), ptr(p), nf)
    out.update(fil_force=ff.copy(), fil_tan=tt.copy())
    # hash -> sort -> reorder -> collide
    h = np.empty(nb, np.uint32)
    idx = np.empty(nb, np.uint32)
    R.ref_calc_hash(C.byref(cfg), None, ptr(h), ptr(idx), ptr(p), nb, 0)
    order = np.argsort(h, kind="stable").astype(np.uint32)
    sh, si = h[order].copy(), idx[order].copy()
    ncell = cfg.n_cells
    cs = np.empty(ncell, np.uint32)
    ce = np.full(ncell, 0xFFFFFFFF, np.uint32)
    sp, sv, st = (np.empty((nb, 4), np.float32) for _ in range(3))
    R.ref_reorder(C.byref(cfg), ptr(cs), ptr(ce), ptr(sp), ptr(sv), ptr(st), ptr(sh), ptr(si), ptr(p), ptr(v), ptr(tt),
                  nb, ncell)
    cf = ff.copy()
    R.ref_collide_filaments(C.byref(cfg), ptr(cf), ptr(sp), ptr(sv), ptr(st), ptr(si), ptr(cs), ptr(ce), nb)
    out.update(hash=h, sorted_hash=sh, sorted_index=si, cell_start=cs, cell_end=ce, sorted_pos=sp, sorted_vel=sv,
               sorted_tan=st, collide_force=cf)
    return out


def srd_case(seed: int, grid, nf: int, L: int):
    R = orc.ref_modern()
    cfg = abi.default_config(abi.NW_MODEL_REF_DEM, nf, L, grid, True)
    cfg.bond_r0 = 0.8
    pos, vel, _ = reference_reset(cfg)
    rng = np.random.default_rng(seed)
    nb, ns = cfg.n_beads, cfg.n_solvent
    n = nb + ns
    shift = (rng.random(3).astype(np.float32) * np.array(cfg.srd_cell_size, np.float32))
    shift[2] = 0.0
    uni = rng.random(cfg.n_srd_cells).astype(np.float32)
    dt_srd = np.float32(0.005 * cfg.srd_gap)
    out = dict(cfg=cfg_bytes(cfg), pos_in=pos.copy(), vel_in=vel.copy(), shift=shift, uniform=uni, dt_srd=dt_srd)
    p, v = pos.copy(), vel.copy()
    h = np.empty(n, np.uint32)
    idx = np.empty(n, np.uint32)
    R.ref_calc_hash(C.byref(cfg), ptr(shift), ptr(h), ptr(idx), ptr(p), n, 1)
    order = np.argsort(h, kind="stable").astype(np.uint32)
    sh, si = h[order].copy(), idx[order].copy()
    ncell = cfg.n_cells
    cs = np.empty(ncell, np.uint32)
    ce = np.full(ncell, 0xFFFFFFFF, np.uint32)
    sp, sv = np.empty((n, 4), np.float32), np.empty((n, 4), np.float32)
    R.ref_reorder(C.byref(cfg), ptr(cs), ptr(ce), ptr(sp), ptr(sv), None, ptr(sh), ptr(si), ptr(p), ptr(v), None, n,
                  ncell)
    nsc = cfg.n_srd_cells
    R.ref_srd_thermostat(C.byref(cfg), ptr(v), ptr(sv), ptr(cs), ptr(ce), ptr(si), nsc)
    thermo_vel = v.copy()
    com = np.zeros((nsc, 4), np.float32)
    R.ref_srd_com(C.byref(cfg), ptr(com), ptr(sv), ptr(cs), ptr(ce), ptr(si), nsc)
    R.ref_collide_solvent(C.byref(cfg), ptr(shift), ptr(p), ptr(v), ptr(com), ptr(uni), n)
    coll_vel = v.copy()
    R.ref_integrate_solvent(C.byref(cfg), ptr(p), ptr(v), float(dt_srd), nb, ns)
    out.update(hash=h, sorted_index=si, cell_start=cs[:nsc], cell_end=ce[:nsc], thermo_vel=thermo_vel, com=com,
               coll_vel=coll_vel, pos_out=p, vel_out=v)
    return out


def wca_case(seed: int):
    A = orc.ref_archived()
    cfg = wca_config(36, 10, (30.0, 30.0), seed=seed)
    pos, vel = initial_state(cfg, seed=seed)
    rng = np.random.default_rng(seed + 100)
    nb = cfg.n_beads
    pos[:, :2] += rng.normal(0.0, 0.03, (nb, 2)).astype(np.float32)
    noise = rng.normal(0.0, 1.0, (nb, 4)).astype(np.float32)
    noise_scale = np.float32(np.sqrt(2.0 * cfg.gamma * cfg.kT / cfg.dt))
    f = np.zeros((nb, 4), np.float32)
    rc = A.ref_archived_forces(C.byref(cfg), ptr(pos), ptr(vel), ptr(noise), float(noise_scale), ptr(f))
    assert rc == 0
    f0 = np.zeros((nb, 4), np.float32)
    v0 = np.zeros_like(vel)
    rc = A.ref_archived_forces(C.byref(cfg), ptr(pos), ptr(v0), None, 0.0, ptr(f0))
    assert rc == 0
    k = np.zeros(7, np.float32)
    A.ref_archived_lj_constants(1.0, 1.0, ptr(k))
    return dict(cfg=cfg_bytes(cfg), pos=pos, vel=vel, noise=noise, noise_scale=noise_scale, force_total=f,
                force_conservative=f0, lj_constants=k)


def main():
    if not orc.have_reference():
        raise SystemExit("reference emulation not built (oracle/_ref); run the build where the reference tree exists")
    np.savez_compressed(HERE / "ref_dem_2d.npz", **ref_dem_case(11, (32, 32, 1), 60, 10))
    np.savez_compressed(HERE / "ref_dem_3d_walls.npz", **ref_dem_case(12, (16, 16, 8), 40, 8, (1, 2, 1)))
    np.savez_compressed(HERE / "ref_srd_2d.npz", **srd_case(13, (32, 32, 1), 30, 10))
    np.savez_compressed(HERE / "wca_archived_2d.npz", **wca_case(14))
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
