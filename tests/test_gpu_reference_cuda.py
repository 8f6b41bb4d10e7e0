"""The reference's own CUDA build on the GPU against libnwgb, on the same inputs.

The reference's kernels (simulation/particles_kernel_impl.cuh, built unmodified
for sm_103a; oracle/ref_cuda) and libnwgb's implementation of the reference's
20 C-ABI symbols (include/nw_legacy.h) run the reference's update sequence
(simulation/particleSystem.cpp:249-413) on identical buffers: force and old
force zeroed, and the same Langevin noise, SRD grid shift and rotation
uniforms injected into both (the reference draws them from cuRAND).

Tolerances: hash, sort order and cell bounds bit-exact; per bead (tests/
parity.py) forces within 1e-5 of the force scale, velocities and tangents
1e-5 relative, positions 1e-5 of the displacement.  Each stage is also
checked against the FP32 oracle, which pins the oracle to the reference's
GPU binary (nvcc contracts multiply-adds; the oracle does not).

Workload of the bead pipeline: the reference-feasible stand-in of the
4,000-bead workload, 400 filaments x 10 beads on a 128 x 128 x 1 grid of unit
cells (power-of-two, as the reference's hash requires), bond 0.8, k_bond 57,
k_bend 10, activity 0.5, gamma 2, kT 0.1, dt 0.005, periodic x / y, wall z.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from nwgb import abi
from nwgb.init import reference_reset
from nwgb.legacy import SimParams, SolventParams
from parity import TOL, force_err, update_err, vec_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    import ref_cuda

    why = ref_cuda.available()
    if why:
        pytest.fail(f"reference CUDA build missing: {why}")
    ref_cuda.lib()
    return ref_cuda


def stand_in_config(lib, M=400, L=10, grid=(128, 128, 1), srd=False):
    """The reference-feasible stand-in configuration (REF_DEM semantics)."""
    cfg = abi.default_config(abi.NW_MODEL_REF_DEM, M, L, grid, srd, lib)
    cfg.bond_r0 = 0.8
    cfg.bond_k = 57.0
    cfg.bend_k = 10.0
    cfg.activity = 0.5
    cfg.kT = 0.1
    cfg.srd_kT = 0.1
    cfg.gamma = 2.0
    cfg.dt = 0.005
    cfg.boundary[0] = abi.NW_PERIODIC
    cfg.boundary[1] = abi.NW_PERIODIC
    cfg.boundary[2] = abi.NW_WALL
    return cfg


def dev(a, dtype=None):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a if dtype is None else np.asarray(a, dtype))).cuda()


def host(t):
    import torch

    torch.cuda.synchronize()
    return t.cpu().numpy()


def P(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class Bufs:
    """The reference's ParticleSystem device buffers for one implementation."""

    def __init__(self, pos, vel, tan, nb, ncells):
        import torch

        n = pos.shape[0]
        self.pos, self.vel, self.tan = dev(pos), dev(vel), dev(tan)
        z = np.zeros((nb, 4), np.float32)
        self.force, self.force_old = dev(z), dev(z)
        self.spos = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        self.svel = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        self.stan = torch.zeros((nb, 4), dtype=torch.float32, device="cuda")
        self.hash = torch.zeros(n, dtype=torch.int32, device="cuda")
        self.index = torch.zeros(n, dtype=torch.int32, device="cuda")
        self.cs = torch.zeros(ncells, dtype=torch.int32, device="cuda")
        self.ce = torch.zeros(ncells, dtype=torch.int32, device="cuda")


class NwgbFns:
    """libnwgb's legacy symbols, called like the reference's."""

    def __init__(self, lib):
        self.lib = lib

    def set_params(self, cfg, shift=(0.0, 0.0, 0.0)):
        from nwgb.legacy import set_parameters

        set_parameters(self.lib, cfg, shift)

    def __getattr__(self, name):
        return getattr(self.lib, name)

    def langevin_apply(self, f, v, g, n):
        self.lib.nw_legacy_langevin_apply(f, v, g, n)

    def collide_solvent_apply(self, p, v, com, u, n):
        self.lib.nw_legacy_collide_solvent_apply(p, v, com, u, n)


class RefFns:
    """The reference's own kernels through the harness."""

    def __init__(self, ref_cuda):
        self.R = ref_cuda.Ref()

    def set_params(self, cfg, shift=(0.0, 0.0, 0.0)):
        self.R.setParameters(SimParams.from_config(cfg))
        self.R.setSolventParameters(SolventParams.from_config(cfg, shift))

    def __getattr__(self, name):
        return getattr(self.R, name)

    def langevin_apply(self, f, v, g, n):
        self.R.langevin_apply(f, v, g, n)

    def collide_solvent_apply(self, p, v, com, u, n):
        self.R.collide_solvent_apply(p, v, com, u, n)


def bead_update(F, B, cfg, noise, record=None):
    """ParticleSystem::update without the SRD sub-step (particleSystem.cpp:
    249-326), with the Langevin noise given instead of drawn."""
    nb, M, ncell = cfg.n_beads, cfg.num_filaments, cfg.n_cells
    F.set_params(cfg)
    F.integrateFilaments(P(B.pos), P(B.vel), P(B.force), P(B.force_old), cfg.dt, nb)
    if record is not None:
        record["int_pos"], record["int_vel"] = host(B.pos)[:nb], host(B.vel)[:nb]
    g = dev(noise)
    F.langevin_apply(P(B.force), P(B.vel), P(g), nb)
    if record is not None:
        record["lang_force"] = host(B.force)
    F.filamentForces(P(B.force), P(B.tan), P(B.pos), float(M))
    if record is not None:
        record["fil_force"], record["fil_tan"] = host(B.force), host(B.tan)
    F.calcHash(P(B.hash), P(B.index), P(B.pos), nb, False)
    if record is not None:
        record["hash"] = host(B.hash).view(np.uint32).copy()
    F.sortParticles(P(B.hash), P(B.index), nb)
    F.reorderDataAndFindCellStart(P(B.cs), P(B.ce), P(B.spos), P(B.svel), P(B.stan), P(B.hash), P(B.index),
                                  P(B.pos), P(B.vel), P(B.tan), nb, ncell)
    if record is not None:
        record["sorted_index"] = host(B.index)[:nb].view(np.uint32).copy()
        record["cell_start"] = host(B.cs).view(np.uint32).copy()
        record["cell_end"] = host(B.ce).view(np.uint32).copy()
    F.collideFilaments(P(B.force), P(B.spos), P(B.svel), P(B.stan), P(B.index), P(B.cs), P(B.ce), nb, ncell)
    if record is not None:
        record["force"] = host(B.force)
    del g


def initial(cfg, seed=4):
    pos, vel, tan = reference_reset(cfg)
    rng = np.random.default_rng(seed)
    pos[:cfg.n_beads, :2] += rng.normal(0, 0.05, (cfg.n_beads, 2)).astype(np.float32)
    return pos, vel, tan


def noise_for(cfg, step, seed=11):
    rng = np.random.default_rng(seed + step)
    sd = np.float32(np.sqrt(np.float32(2.0) * np.float32(cfg.gamma) * np.float32(cfg.kT)))
    z = np.zeros((cfg.n_beads, 4), np.float32)
    z[:, :3] = (rng.standard_normal((cfg.n_beads, 3)) * sd).astype(np.float32)
    return z


def periodic_box(cfg):
    return np.array([cfg.box[a] if cfg.boundary[a] == abi.NW_PERIODIC else 0.0 for a in range(3)])


def test_reference_kernels_load_with_the_reference_layout(ref):
    """The fatbin's __constant__ parameter blocks have this library's struct
    sizes (checked by the harness on load) and every kernel resolves."""
    assert ref.lib() is not None


def test_bead_update_matches_reference_cuda(lib, orc, ref):
    """Five updates of the stand-in workload, stage by stage on the first:
    libnwgb against the reference's GPU kernels, and both against the oracle."""
    cfg = stand_in_config(lib)
    nb = cfg.n_beads
    pos, vel, tan = initial(cfg)
    A = Bufs(pos, vel, tan, nb, cfg.n_cells)
    Bb = Bufs(pos, vel, tan, nb, cfg.n_cells)
    mine, theirs = NwgbFns(lib), RefFns(ref)
    box = periodic_box(cfg)
    for step in range(5):
        noise = noise_for(cfg, step)
        ra, rb = {}, {}
        st = dict(pos=host(Bb.pos)[:nb], vel=host(Bb.vel)[:nb], force=host(Bb.force), force_old=host(Bb.force_old),
                  tangent=host(Bb.tan))
        p_before = st["pos"]
        bead_update(mine, A, cfg, noise, ra)
        bead_update(theirs, Bb, cfg, noise, rb)
        for k in ("hash", "sorted_index", "cell_start"):
            assert np.array_equal(ra[k], rb[k]), (step, k)
        ne = rb["cell_start"] != abi.EMPTY
        assert np.array_equal(ra["cell_end"][ne], rb["cell_end"][ne]), step
        assert update_err(ra["int_pos"], rb["int_pos"], p_before, box) < TOL, step
        assert vec_err(ra["int_vel"], rb["int_vel"]) < TOL, step
        assert vec_err(ra["fil_tan"], rb["fil_tan"]) < TOL, step
        o64 = stage_scales(orc, cfg, rb, noise)
        assert force_err(ra["lang_force"], rb["lang_force"], o64["lang"]) < TOL, step
        assert force_err(ra["fil_force"], rb["fil_force"], o64["fil"]) < TOL, step
        assert force_err(ra["force"], rb["force"], o64["pair"]) < TOL, step
        # the FP32 oracle's stages from the reference's own inputs
        o32 = oracle_stages(orc, cfg, st, noise, rb)
        assert np.array_equal(o32["hash"], rb["hash"]), step
        assert update_err(o32["int_pos"], rb["int_pos"], p_before, box) < TOL, step
        assert force_err(o32["force"], rb["force"], o64["pair"]) < TOL, step


def stage_scales(orc, cfg, rb, noise):
    """Force scales of the three force stages of an update, from the FP64
    oracle on the reference's own intermediate arrays."""
    nb = cfg.n_beads
    out = {}
    with orc.force_scale(nb) as S:
        orc.langevin(cfg, np.zeros((nb, 4), np.float32), rb["int_vel"], noise, prec=64)
    out["lang"] = S.values[:nb].copy()
    with orc.force_scale(nb) as S:
        orc.filament(cfg, rb["lang_force"], rb["fil_tan"], rb["int_pos"], prec=64)
    out["fil"] = out["lang"] + S.values[:nb]
    with orc.force_scale(nb) as S:
        orc.pair(cfg, rb["fil_force"], rb["int_pos"], rb["int_vel"], rb["fil_tan"], rb["sorted_index"],
                 rb["cell_start"], rb["cell_end"], prec=64)
    out["pair"] = out["fil"] + S.values[:nb]
    return out


def oracle_stages(orc, cfg, st, noise, rb):
    """The FP32 oracle's integrate, hash and pair force from the same inputs."""
    p, v, f, fo = orc.integrate(cfg, st["pos"], st["vel"], st["force"], st["force_old"], cfg.dt, prec=32)
    h, _ = orc.calc_hash(cfg, p)
    fp = orc.pair(cfg, rb["fil_force"], rb["int_pos"], rb["int_vel"], rb["fil_tan"], rb["sorted_index"],
                  rb["cell_start"], rb["cell_end"], prec=32)
    return dict(int_pos=p, hash=h, force=fp)


def test_srd_pipeline_matches_reference_cuda(lib, orc, ref):
    """The reference's SRD sub-step (particleSystem.cpp:341-413) on a small
    stand-in (64 x 64 bead cells, 32 x 32 SRD cells of side 2, 10 solvent per
    SRD cell), with the grid shift and the per-cell rotation uniforms injected."""
    import torch

    cfg = stand_in_config(lib, M=150, L=10, grid=(64, 64, 1), srd=True)
    nb, ns = cfg.n_beads, cfg.n_solvent
    n = nb + ns
    assert cfg.n_srd_cells <= 4 * nb
    pos, vel, tan = initial(cfg)
    rng = np.random.default_rng(5)
    shift = (float(np.float32(rng.uniform(0, 2))), float(np.float32(rng.uniform(0, 2))), 0.0)
    uni = rng.uniform(0, 1, cfg.n_srd_cells).astype(np.float32)
    res = []
    for F in (NwgbFns(lib), RefFns(ref)):
        B = Bufs(pos, vel, tan, nb, cfg.n_cells)
        com = torch.zeros((cfg.n_srd_cells, 4), dtype=torch.float32, device="cuda")
        u = dev(uni)
        F.set_params(cfg, shift)
        F.calcHash(P(B.hash), P(B.index), P(B.pos), n, True)
        F.sortParticles(P(B.hash), P(B.index), n)
        F.reorderDataAndFindCellStart(P(B.cs), P(B.ce), P(B.spos), P(B.svel), None, P(B.hash), P(B.index),
                                      P(B.pos), P(B.vel), None, n, cfg.n_cells)
        r = dict(hash=host(B.hash).view(np.uint32).copy(), index=host(B.index).view(np.uint32).copy(),
                 cs=host(B.cs).view(np.uint32)[:cfg.n_srd_cells].copy())
        F.solventIsokineticThermostat(P(B.vel), P(B.svel), P(B.cs), P(B.ce), P(B.index), cfg.n_srd_cells)
        r["thermo_vel"] = host(B.vel)
        F.solventCellCentorOfMomentum(P(com), P(B.svel), P(B.cs), P(B.ce), P(B.index), cfg.n_srd_cells)
        r["com"] = host(com)
        F.collide_solvent_apply(P(B.pos), P(B.vel), P(com), P(u), n)
        r["coll_vel"] = host(B.vel)
        r["pre_stream"] = host(B.pos)
        F.integrateSolvent(P(B.pos), P(B.vel), cfg.dt * cfg.srd_gap, nb, ns)
        r["pos"], r["vel"] = host(B.pos), host(B.vel)
        res.append(r)
    a, b = res
    for k in ("hash", "index", "cs"):
        assert np.array_equal(a[k], b[k]), k
    for k in ("thermo_vel", "coll_vel", "vel"):
        assert vec_err(a[k], b[k]) < TOL, k
    assert vec_err(a["com"], b["com"]) < TOL
    assert np.array_equal(a["pos"][:nb], b["pos"][:nb])
    assert update_err(a["pos"][nb:], b["pos"][nb:], b["pre_stream"][nb:], periodic_box(cfg)) < TOL


def test_particle_system_matches_reference_update_loop(lib, ref):
    """The reference's ParticleSystem::update loop on its own kernels (cuRAND
    for the noise, thrust for the sort; kT = 0 so that the noise is zero)
    against this library's ParticleSystem (the reference's host API on the
    handle engine), 20 updates from the same reset state: identical sort
    order, per-bead trajectories to 1e-4 (20 steps of FP32 contraction
    differences)."""
    import nwgb

    cfg = stand_in_config(lib)
    cfg.kT = 0.0
    nb = cfg.n_beads
    pos, vel, tan = initial(cfg)
    rs = ref.RefSystem(SimParams.from_config(cfg))
    rs.set(ref.POS, pos)
    rs.set(ref.VEL, vel)
    rs.set(ref.TANGENT, tan)
    ps = nwgb.ParticleSystem(cfg.num_filaments, cfg.filament_size, tuple(cfg.grid), False, cfg=cfg)
    try:
        ps.setArray(0, pos, 0, nb)
        ps.setArray(1, vel, 0, nb)
        ps.setArray(2, tan, 0, nb)
        for k in range(20):
            rs.update(cfg.dt)
            ps.update(cfg.dt)
            if k == 0:
                a = ps.system.get_array(abi.NW_SORTED_INDEX)
                b = rs.get(ref.INDEX, np.uint32)[:nb]
                assert np.array_equal(a, b)
        pa, va = ps.getArray(0), ps.getArray(1)
        pb, vb = rs.get(ref.POS)[:nb], rs.get(ref.VEL)[:nb]
        assert update_err(pa, pb, pos[:nb], periodic_box(cfg)) < 1e-4
        assert vec_err(va, vb) < 1e-4
        assert rs.update_count == 20
    finally:
        ps.close()
        rs.close()
