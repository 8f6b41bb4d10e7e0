"""Parity of the CUDA step (through the C ABI) with the CPU oracle.

Tolerances (tests/parity.py): cell hashes, sort order and cell bounds
bit-exact; per bead, forces within 1e-5 of the bead's force scale, velocities
and tangents within 1e-5 relative, the one-step position update within 1e-5
of the bead's displacement (up to the final FP32 rounding), against the FP32
oracle; against the FP64 oracle within 1e-5 or the FP32 oracle's own FP64
error, whichever is larger.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from nwgb import abi
from nwgb.init import initial_state, reference_reset, wca_config
from parity import SOLVENT_FLOOR, TOL, force_err, fp64_bound, summary, update_err, vec_err

pytestmark = pytest.mark.gpu


def make_case(kind: str, lib):
    if kind == "wca":
        cfg = wca_config(120, 10, (50.0, 50.0), seed=1, lib=lib)
        pos, vel = initial_state(cfg, seed=1)
        tan = np.zeros((cfg.n_beads, 4), np.float32)
    elif kind == "wca_srd":
        cfg = wca_config(80, 10, (40.0, 40.0), srd=True, seed=2, lib=lib)
        pos, vel = initial_state(cfg, seed=2)
        tan = np.zeros((cfg.n_beads, 4), np.float32)
    elif kind == "wca_srd_dense":
        # 24 solvent per SRD cell: cells take the warp-per-cell collision
        cfg = wca_config(80, 10, (40.0, 40.0), srd=True, srd_density=24.0, seed=6, lib=lib)
        pos, vel = initial_state(cfg, seed=6)
        tan = np.zeros((cfg.n_beads, 4), np.float32)
    elif kind == "wca_srd_rounds":
        # about 9 solvent per SRD cell: warps hold more members than their
        # staging and collide their cells in two or three rounds
        cfg = wca_config(80, 10, (40.0, 40.0), srd=True, srd_density=9.0, seed=7, lib=lib)
        pos, vel = initial_state(cfg, seed=7)
        tan = np.zeros((cfg.n_beads, 4), np.float32)
    elif kind == "wca_srd_packed":
        # about 215 solvent per SRD cell: every cell takes the warp-per-cell
        # collision, which orders up to 384 members exactly
        cfg = wca_config(12, 10, (16.0, 16.0), srd=True, srd_density=215.0, seed=8, lib=lib)
        pos, vel = initial_state(cfg, seed=8)
        tan = np.zeros((cfg.n_beads, 4), np.float32)
    elif kind == "wca_reverse":
        cfg = wca_config(60, 12, (40.0, 40.0), seed=3, lib=lib)
        cfg.reverse_probability = 0.4
        pos, vel = initial_state(cfg, seed=3)
        tan = np.zeros((cfg.n_beads, 4), np.float32)
    elif kind in ("ref", "ref_srd", "ref_walls"):
        srd = kind == "ref_srd"
        cfg = abi.default_config(abi.NW_MODEL_REF_DEM, 150, 10, (64, 64, 1), srd, lib)
        cfg.bond_r0 = 0.8
        cfg.bend_k = 10.0
        cfg.activity = 0.5
        cfg.spring = 57.0
        cfg.kT = 0.1
        cfg.gamma = 2.0
        cfg.srd_kT = 0.1
        cfg.seed = 9
        if kind == "ref_walls":
            cfg.boundary[1] = abi.NW_WALL_NO_SLIP
            cfg.boundary[2] = abi.NW_WALL
        pos, vel, tan = reference_reset(cfg)
        rng = np.random.default_rng(4)
        pos[:cfg.n_beads, :2] += rng.normal(0, 0.05, (cfg.n_beads, 2)).astype(np.float32)
    elif kind in ("ref_strip", "ref_alias"):
        # REF_DEM grids narrower than the pair pass's 32 x 4 cell tiles: a
        # 16 x 8 strip, and 2 x 16 where the x offsets -1 and +1 reach the
        # same cell (the reference then visits it twice)
        M, L, grid = (40, 4, (16, 8, 1)) if kind == "ref_strip" else (10, 2, (2, 16, 1))
        cfg = abi.default_config(abi.NW_MODEL_REF_DEM, M, L, grid, False, lib)
        cfg.bond_r0 = 0.8
        cfg.bend_k = 10.0
        cfg.activity = 0.5
        cfg.spring = 57.0
        cfg.kT = 0.1
        cfg.gamma = 2.0
        cfg.seed = 14
        rng = np.random.default_rng(15)
        pos = np.zeros((cfg.n_beads, 4), np.float32)
        lo = np.array([cfg.origin[0], cfg.origin[1]])
        hi = lo + np.array([cfg.box[0], cfg.box[1]])
        for w in range(M):
            head = rng.uniform(lo + 0.5, hi - 0.5 - np.array([0.0, 0.8 * (L - 1)]))
            for k in range(L):
                pos[w * L + k, :2] = head + np.array([rng.normal(0, 0.05), 0.8 * k])
        pos[:, 3] = cfg.radius
        vel = np.zeros_like(pos)
        vel[:, :2] = rng.normal(0, 0.3, (cfg.n_beads, 2))
        vel[:, 3] = cfg.mass
        tan = np.zeros_like(pos)
        tan[:, 1] = 1.0
    elif kind in ("wca_3d", "ref_3d"):
        # 3D grids: straight worms along x on a jittered y-z lattice of rows
        if kind == "wca_3d":
            cfg = abi.default_config(abi.NW_MODEL_WCA_WORMS, 96, 10, (18, 12, 12), False, lib)
            cfg.dim = 3
            for a in range(3):
                cfg.cell_size[a] = 1.125
            abi.check(lib.nw_config_finalize(C.byref(cfg)))
            cfg.seed = 12
        else:
            cfg = abi.default_config(abi.NW_MODEL_REF_DEM, 96, 10, (32, 16, 16), False, lib)
            # the parameters of the 2D REF_DEM cases
            cfg.bond_r0 = 0.8
            cfg.bend_k = 10.0
            cfg.activity = 0.5
            cfg.spring = 57.0
            cfg.kT = 0.1
            cfg.gamma = 2.0
            cfg.seed = 13
        pos, vel, tan = lattice_3d(cfg, seed=7)
        # off the relaxed lattice, as the 2D REF_DEM cases are
        pos[:, :3] += np.random.default_rng(8).normal(0, 0.05, (cfg.n_beads, 3)).astype(np.float32)
    else:
        raise ValueError(kind)
    return cfg, pos, vel, tan


def lattice_3d(cfg, seed):
    """Worms along x in rows on a y-z lattice (pitch 1.5), jittered; Maxwell-
    Boltzmann velocities in three dimensions."""
    rng = np.random.default_rng(seed)
    M, L = cfg.num_filaments, cfg.filament_size
    org = np.array([cfg.origin[0], cfg.origin[1], cfg.origin[2]])
    box = np.array([cfg.box[0], cfg.box[1], cfg.box[2]])
    length = (L - 1) * cfg.bond_r0
    per_x = int(box[0] // (length + 1.0))
    ny, nz = int(box[1] // 1.5), int(box[2] // 1.5)
    assert per_x * ny * nz >= M
    pos = np.zeros((M * L, 4), np.float32)
    for w in range(M):
        ix, rest = w % per_x, w // per_x
        iy, iz = rest % ny, rest // ny
        head = org + np.array([ix * (length + 1.0) + 0.5, (iy + 0.5) * 1.5, (iz + 0.5) * 1.5])
        head[1:] += rng.normal(0, 0.05, 2)
        beads = head[None, :] + np.arange(L)[:, None] * np.array([cfg.bond_r0, 0.0, 0.0])[None, :]
        pos[w * L:(w + 1) * L, :3] = beads
    pos[:, 3] = cfg.radius
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0, np.sqrt(cfg.kT), (M * L, 3))
    vel[:, 3] = cfg.mass
    return pos, vel, np.zeros_like(pos)


def run_gpu(cfg, pos, vel, tan, nsteps=1, graphs=True, force=None, force_old=None, step=0):
    import nwgb

    s = nwgb.System(cfg)
    s.set_graphs(graphs)
    s.set_array(abi.NW_POSITION, pos)
    s.set_array(abi.NW_VELOCITY, vel)
    s.set_array(abi.NW_TANGENT, tan)
    if force is not None:
        s.set_array(abi.NW_FORCE, force)
        s.set_array(abi.NW_FORCE_OLD, force_old)
    if step:
        s.set_step(step)
    s.step(nsteps, cfg.dt)
    s.sync()
    out = {k: s.get_array(a) for k, a in (("pos", abi.NW_POSITION), ("vel", abi.NW_VELOCITY),
                                           ("force", abi.NW_FORCE), ("force_old", abi.NW_FORCE_OLD),
                                           ("tangent", abi.NW_TANGENT), ("hash", abi.NW_HASH),
                                           ("sorted_index", abi.NW_SORTED_INDEX),
                                           ("cell_start", abi.NW_CELL_START), ("cell_end", abi.NW_CELL_END))}
    out["launches"] = s.last_launch_count
    s.close()
    return out


def run_oracle(orc, cfg, pos, vel, tan, nsteps=1, prec=32, force=None, force_old=None, step=0, force_scale=False):
    z = np.zeros((cfg.n_beads, 4), np.float32)
    st = dict(pos=pos, vel=vel, force=z if force is None else force, force_old=z if force_old is None else force_old,
              tangent=tan)
    for k in range(nsteps):
        st = orc.step(cfg, st, step + k, cfg.dt, prec, force_scale=force_scale and k == nsteps - 1)
    return st


def periodic_box(cfg):
    """Box lengths of the periodic axes (0 for walls): the minimum image of a displacement."""
    return np.array([cfg.box[a] if cfg.boundary[a] == abi.NW_PERIODIC else 0.0 for a in range(3)])


def check_step_parity(cfg, g, o, o64, pos0):
    """Bit-exact integer outputs; per-bead float parity against the FP32 and
    the FP64 oracle (module docstring)."""
    nb = cfg.n_beads
    assert np.array_equal(g["hash"], o["hash"])
    assert np.array_equal(g["sorted_index"], o["sorted_index"])
    assert np.array_equal(g["cell_start"], o["cell_start"])
    ne = o["cell_start"] != abi.EMPTY
    assert np.array_equal(g["cell_end"][ne], o["cell_end"][ne])
    # the old force is the previous step's force, copied by the integrator
    assert np.array_equal(g["force_old"][:, :3], o["force_old"][:, :3])
    S = o64["force_scale"]
    box = periodic_box(cfg)
    metrics = {
        "force": lambda x, y: force_err(x["force"], y["force"], S),
        "vel": lambda x, y: vec_err(x["vel"][:nb], y["vel"][:nb]),
        "tangent": lambda x, y: vec_err(x["tangent"], y["tangent"]),
        "displacement": lambda x, y: update_err(x["pos"][:nb], y["pos"][:nb], pos0[:nb], box),
    }
    for k, m in metrics.items():
        e32 = m(g, o)
        assert e32 < TOL, (k, "fp32", e32, summary(g[k if k != "displacement" else "pos"], o[k if k != "displacement" else "pos"]))
        e64 = m(g, o64)
        assert e64 < fp64_bound(m(o, o64)), (k, "fp64", e64, m(o, o64))


CASES = ["wca", "wca_srd", "wca_srd_dense", "wca_srd_rounds", "wca_srd_packed", "wca_reverse", "wca_3d", "ref", "ref_srd",
         "ref_walls", "ref_3d", "ref_strip", "ref_alias"]
STRATEGIES = [abi.NW_STRATEGY_CELL_LISTS, abi.NW_STRATEGY_SORTED, abi.NW_STRATEGY_VERLET]
# launches of one update: (bead step, SRD collision) + the step counter; Verlet systems
# add the on-demand cell-list kernel
LAUNCHES = {abi.NW_STRATEGY_CELL_LISTS: (2, 7), abi.NW_STRATEGY_SORTED: (6, 7), abi.NW_STRATEGY_VERLET: (3, 7)}


def strategy_applies(kind, strategy):
    # Verlet lists serve the WCA law only (the REF_DEM pair set is cell-based)
    return not (strategy == abi.NW_STRATEGY_VERLET and kind.startswith("ref"))


@pytest.mark.parametrize("strategy", STRATEGIES)
@pytest.mark.parametrize("kind", CASES)
def test_one_step_matches_oracle(lib, orc, kind, strategy):
    """Step 0 from rest forces (f = f_old = 0): hashes, sort and cell bounds,
    the forces of the step, tangents, and the SRD collision of step 0."""
    if not strategy_applies(kind, strategy):
        pytest.skip("Verlet lists are WCA-only")
    cfg, pos, vel, tan = make_case(kind, lib)
    cfg.strategy = strategy
    g = run_gpu(cfg, pos, vel, tan)
    o = run_oracle(orc, cfg, pos, vel, tan, 1, 32)
    o64 = run_oracle(orc, cfg, pos, vel, tan, 1, 64, force_scale=True)
    check_step_parity(cfg, g, o, o64, pos)
    nb = cfg.n_beads
    bead, srd = LAUNCHES[strategy]
    if cfg.srd_enabled:  # solvent after the collision of step 0, particle by particle
        box = periodic_box(cfg)
        before = ref_streamed_from(o, cfg)
        sv = lambda x, y: vec_err(x["vel"][nb:], y["vel"][nb:], SOLVENT_FLOOR)  # noqa: E731
        sp = lambda x, y: update_err(x["pos"][nb:], y["pos"][nb:], before, box, SOLVENT_FLOOR)  # noqa: E731
        for m in (sv, sp):
            assert m(g, o) < TOL, m(g, o)
            assert m(g, o64) < fp64_bound(m(o, o64)), (m(g, o64), m(o, o64))
        assert g["launches"] == bead + srd + 1
    else:
        assert g["launches"] == bead + 1


def ref_streamed_from(ref, cfg):
    """Solvent positions before the streaming of the collision that ends the
    step: the streamed position minus velocity x srd_gap x dt."""
    nb = cfg.n_beads
    p = np.asarray(ref["pos"][nb:], np.float64)[:, :3]
    v = np.asarray(ref["vel"][nb:], np.float64)[:, :3]
    return p - v * (cfg.srd_gap * cfg.dt)


@pytest.mark.parametrize("strategy", STRATEGIES)
@pytest.mark.parametrize("kind", [c for c in CASES if "srd" not in c or c == "wca_srd"] + ["ref_srd"])
def test_update_from_forced_state_matches_oracle(lib, orc, kind, strategy):
    """Step 1 from the oracle's state after step 0 (non-zero f and f_old): the
    velocity-Verlet update v += (f + f_old) dt / 2, r += v dt + f dt^2 / 2 of
    every bead, then the next forces, per bead against FP32 and FP64."""
    if not strategy_applies(kind, strategy):
        pytest.skip("Verlet lists are WCA-only")
    cfg, pos, vel, tan = make_case(kind, lib)
    cfg.strategy = strategy
    s1 = run_oracle(orc, cfg, pos, vel, tan, 1, 32)
    nb = cfg.n_beads
    assert np.abs(s1["force"][:, :3]).max() > 0 and np.abs(s1["force_old"]).max() == 0
    st = dict(pos=s1["pos"], vel=s1["vel"], tan=s1["tangent"], force=s1["force"], force_old=s1["force_old"])
    g = run_gpu(cfg, st["pos"], st["vel"], st["tan"], force=st["force"], force_old=st["force_old"], step=1)
    o = run_oracle(orc, cfg, st["pos"], st["vel"], st["tan"], 1, 32, force=st["force"], force_old=st["force_old"],
                   step=1)
    o64 = run_oracle(orc, cfg, st["pos"], st["vel"], st["tan"], 1, 64, force=st["force"],
                     force_old=st["force_old"], step=1, force_scale=True)
    check_step_parity(cfg, g, o, o64, st["pos"])


@pytest.mark.parametrize("strategy", STRATEGIES)
@pytest.mark.parametrize("kind", ["wca", "ref_srd", "wca_srd_dense"])
def test_graph_replay_is_bit_identical_to_direct_launches(lib, kind, strategy):
    if not strategy_applies(kind, strategy):
        pytest.skip("Verlet lists are WCA-only")
    cfg, pos, vel, tan = make_case(kind, lib)
    cfg.strategy = strategy
    a = run_gpu(cfg, pos, vel, tan, nsteps=12, graphs=True)
    b = run_gpu(cfg, pos, vel, tan, nsteps=12, graphs=False)
    c = run_gpu(cfg, pos, vel, tan, nsteps=12, graphs=True)
    for k in ("pos", "vel", "force", "tangent", "sorted_index"):
        assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(a[k], c[k]), k  # run twice: no races


@pytest.mark.parametrize("graphs", [True, False])
@pytest.mark.parametrize("strategy", STRATEGIES)
def test_run_split_over_calls_is_bit_identical(lib, strategy, graphs):
    """25 updates with SRD collisions at 0, 10 and 20 in one call, in three
    calls of other SRD phases, and in three calls with the positions written
    back from the host in between, give the same state bit for bit."""
    import nwgb

    cfg, pos, vel, tan = make_case("wca_srd", lib)
    cfg.strategy = strategy

    def run(splits, rewrite):
        s = nwgb.System(cfg)
        s.set_graphs(graphs)
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.set_array(abi.NW_TANGENT, tan)
        for n in splits:
            if rewrite:
                s.set_array(abi.NW_POSITION, s.get_array(abi.NW_POSITION))
            s.step(n, cfg.dt)
        s.sync()
        out = (s.get_array(abi.NW_POSITION), s.get_array(abi.NW_VELOCITY))
        s.close()
        return out

    a = run([25], False)
    assert len(a[0]) > cfg.n_beads
    for x in (run([7, 9, 9], False), run([7, 9, 9], True)):
        assert np.array_equal(a[0], x[0]) and np.array_equal(a[1], x[1])


@pytest.mark.parametrize("strategy", STRATEGIES)
def test_planar_system_carries_z(lib, strategy):
    """Two-dimensional WCA worms compute in the xy plane, with the two vector
    components of the archived worm kernels: beads given z offsets and z
    velocities follow the same xy trajectory bit for bit, keep their z and z
    velocity, and take no z force."""
    cfg, pos, vel, tan = make_case("wca", lib)
    assert cfg.dim == 2 and cfg.model == abi.NW_MODEL_WCA_WORMS
    cfg.strategy = strategy
    a = run_gpu(cfg, pos, vel, tan, nsteps=12)
    rng = np.random.default_rng(3)
    pz, vz = pos.copy(), vel.copy()
    pz[:, 2] = rng.uniform(-0.4, 0.4, len(pz)).astype(np.float32)  # inside the z extent: no wrap
    vz[:, 2] = rng.normal(0.0, 0.5, len(vz)).astype(np.float32)
    b = run_gpu(cfg, pz, vz, tan, nsteps=12)
    for k in ("pos", "vel", "force", "force_old"):
        assert np.array_equal(a[k][:, :2], b[k][:, :2]), k
    assert np.array_equal(b["pos"][:, 2], pz[:, 2])
    assert np.array_equal(b["vel"][:, 2], vz[:, 2])
    assert np.all(b["force"][:, 2] == 0) and np.all(b["force_old"][:, 2] == 0)


@pytest.mark.parametrize("kind", ["wca", "wca_srd", "ref"])
def test_strategies_agree(lib, orc, kind):
    """Cell lists visit each cell's beads in index order, as the sorted
    arrays do: both strategies give the same cell assignment and sort order
    and the same trajectory up to FP32 contraction differences of the two
    kernel codes."""
    cfg, pos, vel, tan = make_case(kind, lib)
    out = []
    for strategy in STRATEGIES:
        if strategy_applies(kind, strategy):
            cfg.strategy = strategy
            out.append(run_gpu(cfg, pos, vel, tan, nsteps=15, graphs=True))
    nb = cfg.n_beads
    S = run_oracle(orc, cfg, pos, vel, tan, 15, 64, force_scale=True)["force_scale"]
    box = periodic_box(cfg)
    for o in out[1:]:
        for k in ("hash", "sorted_index", "cell_start"):
            assert np.array_equal(out[0][k], o[k]), k
        # 15 steps of the same dynamics; the strategies sum pair forces in
        # different orders, and those FP32 differences grow along the trajectory
        assert update_err(o["pos"][:nb], out[0]["pos"][:nb], pos[:nb], box) < 1e-4
        assert vec_err(o["vel"][:nb], out[0]["vel"][:nb]) < 1e-4
        assert vec_err(o["tangent"], out[0]["tangent"]) < 1e-4
        for k in ("force", "force_old"):
            assert force_err(o[k], out[0][k], S) < 1e-4, k


@pytest.mark.parametrize("skin", [0.02, 0.3, 1.0])
def test_verlet_lists_track_oracle_across_rebuilds(lib, orc, skin):
    """A hot WCA system (kT = 2) moves far enough that lists are rebuilt
    several times in 40 steps for the small skins and reused for the large
    one; every step's forces must stay those of the full cell scan."""
    cfg, pos, vel, tan = make_case("wca", lib)
    cfg.kT = 2.0
    cfg.strategy = abi.NW_STRATEGY_VERLET
    cfg.neighbor_skin = skin
    n = 40
    g = run_gpu(cfg, pos, vel, tan, nsteps=n)
    cfg.strategy = abi.NW_STRATEGY_SORTED
    s = run_gpu(cfg, pos, vel, tan, nsteps=n)
    # same dynamics as the reference-order path up to FP32 summation order,
    # amplified over 40 steps of a hot (kT = 2) system
    box = periodic_box(cfg)
    S = run_oracle(orc, cfg, pos, vel, tan, n, 64, force_scale=True)["force_scale"]
    assert update_err(g["pos"], s["pos"], pos, box) < 1e-4
    assert force_err(g["force"], s["force"], S) < 1e-4
    # the reference-grid hash of the Verlet system is computed when read
    assert np.mean(g["hash"] == s["hash"]) > 0.999


def test_verlet_list_overflow_is_reported(lib):
    import nwgb

    cfg, pos, vel, tan = make_case("wca", lib)
    cfg.strategy = abi.NW_STRATEGY_VERLET
    cfg.neighbor_capacity = 4
    cfg.neighbor_skin = 3.0  # ~30 beads within the list radius
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.step(1, cfg.dt)
        with pytest.raises(nwgb.NwError) as e:
            s.sync()
        assert e.value.status == abi.NW_ERR_CELL_OVERFLOW


@pytest.mark.parametrize("kind", ["wca", "wca_srd", "ref"])
def test_short_trajectory_tracks_oracle(lib, orc, kind):
    cfg, pos, vel, tan = make_case(kind, lib)
    n = 12
    g = run_gpu(cfg, pos, vel, tan, nsteps=n)
    o = run_oracle(orc, cfg, pos, vel, tan, n, 32)
    nb = cfg.n_beads
    # trajectories separate only by accumulated FP32 rounding over 12 steps
    o64 = run_oracle(orc, cfg, pos, vel, tan, n, 64, force_scale=True)
    box = periodic_box(cfg)
    assert update_err(g["pos"][:nb], o["pos"][:nb], pos[:nb], box) < 1e-4
    assert vec_err(g["vel"][:nb], o["vel"][:nb]) < 1e-4
    assert force_err(g["force"], o["force"], o64["force_scale"]) < 1e-4
    assert np.mean(g["sorted_index"] == o["sorted_index"]) > 0.999


def test_checkpoint_resume_is_bit_exact(lib):
    import nwgb

    cfg, pos, vel, tan = make_case("wca_srd", lib)
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.step(7, cfg.dt)
        blob = s.checkpoint()
        s.step(9, cfg.dt)
        ref = s.get_array(abi.NW_POSITION)
    with nwgb.System(cfg) as s2:
        s2.restore(blob)
        assert s2.step_index == 7
        s2.step(9, cfg.dt)
        assert np.array_equal(s2.get_array(abi.NW_POSITION), ref)


def test_nonfinite_state_is_reported(lib):
    import nwgb

    cfg, pos, vel, tan = make_case("wca", lib)
    pos = pos.copy()
    pos[17, 0] = np.nan
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.step(1, cfg.dt)
        with pytest.raises(nwgb.NwError) as e:
            s.sync()
        assert e.value.status == abi.NW_ERR_NONFINITE
        # the context stays usable: a clean state steps without error
        p2, _ = initial_state(cfg, seed=1)
        s.set_array(abi.NW_POSITION, p2)
        s.zero_forces()
        s.step(2, cfg.dt)
        s.sync()


def test_empty_system_steps(lib):
    import nwgb

    cfg = wca_config(0, 10, (20.0, 20.0), lib=lib)
    with nwgb.System(cfg) as s:
        s.step(3, cfg.dt)
        s.sync()
        assert s.step_index == 3


@pytest.mark.parametrize("strategy", STRATEGIES)
def test_round_trip_per_step_matches_synchronous(lib, strategy):
    """Positions and velocities fed from and read back to pinned host memory
    around every single step (12 steps, a collision at step 10), as the
    end-to-end loop does: the asynchronous reads, which start once the step's
    positions and velocities are final, equal the synchronous path bit for
    bit; an asynchronous read after the positions were set returns the set
    values."""
    import nwgb
    import torch

    cfg, pos, vel, tan = make_case("wca_srd", lib)
    cfg.strategy = strategy
    nb = cfg.n_beads
    out = []
    for use_async in (False, True):
        with nwgb.System(cfg) as s:
            s.set_array(abi.NW_POSITION, pos)
            s.set_array(abi.NW_VELOCITY, vel)
            hp = torch.from_numpy(pos[:nb].copy()).pin_memory().numpy()
            hv = torch.from_numpy(vel[:nb].copy()).pin_memory().numpy()
            for _ in range(12):
                if use_async:
                    s.set_array_async(abi.NW_POSITION, hp)
                    s.set_array_async(abi.NW_VELOCITY, hv)
                    s.step(1, cfg.dt)
                    s.get_array_async(abi.NW_POSITION, hp)
                    s.get_array_async(abi.NW_VELOCITY, hv)
                    s.sync()
                else:
                    s.set_array(abi.NW_POSITION, hp)
                    s.set_array(abi.NW_VELOCITY, hv)
                    s.step(1, cfg.dt)
                    s.sync()
                    hp[:] = s.get_array(abi.NW_POSITION, 0, nb)
                    hv[:] = s.get_array(abi.NW_VELOCITY, 0, nb)
            out.append((hp.copy(), hv.copy(), s.get_array(abi.NW_POSITION)))
            if use_async:
                moved = hp.copy()
                moved[:, 0] += 0.01
                back = torch.from_numpy(np.zeros_like(moved)).pin_memory().numpy()
                s.set_array(abi.NW_POSITION, moved)
                s.get_array_async(abi.NW_POSITION, back)
                s.sync()
                assert np.array_equal(back, moved)
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def test_async_copies_match_synchronous(lib):
    """nw_set_array_async / nw_get_array_async enqueue the same copies as the
    synchronous calls: one step fed and read back through them equals the
    synchronous path bit for bit."""
    import nwgb
    import torch

    cfg, pos, vel, tan = make_case("wca_srd", lib)
    out = []
    for use_async in (False, True):
        with nwgb.System(cfg) as s:
            if use_async:
                hp = torch.from_numpy(pos.copy()).pin_memory().numpy()
                hv = torch.from_numpy(vel.copy()).pin_memory().numpy()
                s.set_array_async(abi.NW_POSITION, hp)
                s.set_array_async(abi.NW_VELOCITY, hv)
                s.step(3, cfg.dt)
                s.get_array_async(abi.NW_POSITION, hp)
                s.get_array_async(abi.NW_VELOCITY, hv)
                s.sync()
                out.append((hp.copy(), hv.copy()))
            else:
                s.set_array(abi.NW_POSITION, pos)
                s.set_array(abi.NW_VELOCITY, vel)
                s.step(3, cfg.dt)
                s.sync()
                out.append((s.get_array(abi.NW_POSITION), s.get_array(abi.NW_VELOCITY)))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
