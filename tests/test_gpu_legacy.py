"""The reference's 20 C-ABI symbols, as implemented by libnwgb.so, against the
golden vectors of the reference's own kernels (tests/golden) and the oracle.

Device buffers come from torch (memory plumbing only); every call goes
through the library's extern "C" entry points.  Tolerance: bit-exact for
hashes, sort order and cell bounds; per bead 1e-5 for floats (tests/parity.py:
forces against the FP64 oracle's force scale of the same call, velocities and
tangents relative, positions relative to the bead's displacement).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN
from nwgb.abi import NwConfig
from parity import force_err, update_err, vec_err

pytestmark = pytest.mark.gpu
TOL = 1e-5


def torch_dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch

    torch.cuda.synchronize()
    return t.cpu().numpy()


def ptr(t):
    return C.c_void_p(t.data_ptr())


def load(name):
    d = dict(np.load(GOLDEN / name))
    return NwConfig.from_buffer_copy(d["cfg"].tobytes()), d


def set_legacy_params(lib, cfg: NwConfig, shift=(0.0, 0.0, 0.0)):
    """Fill the reference's SimParams / SolventParams from a configuration."""
    from nwgb.legacy import set_parameters

    return set_parameters(lib, cfg, shift)


def norms(a):
    return np.linalg.norm(np.asarray(a, np.float64)[:, :3], axis=1)


def box_of(cfg):
    return np.array([cfg.box[a] if cfg.boundary[a] == 0 else 0.0 for a in range(3)])


@pytest.mark.parametrize("name", ["ref_dem_2d.npz", "ref_dem_3d_walls.npz"])
def test_legacy_bead_pipeline_matches_reference(lib, orc, name):
    cfg, d = load(name)
    set_legacy_params(lib, cfg)
    nb = cfg.n_beads
    p, v = torch_dev(d["pos_in"]), torch_dev(d["vel_in"])
    f, fo = torch_dev(d["force_in"]), torch_dev(d["force_old_in"])
    lib.integrateFilaments(ptr(p), ptr(v), ptr(f), ptr(fo), float(d["dt"]), nb)
    assert update_err(host(p), d["int_pos"], d["pos_in"], box_of(cfg)) < TOL
    assert vec_err(host(v), d["int_vel"]) < TOL
    assert np.array_equal(host(f), d["int_force"]) and np.array_equal(host(fo), d["int_force_old"])
    # Langevin kernel with the injected noise
    noise = torch_dev(d["noise"])
    p, v = torch_dev(d["int_pos"]), torch_dev(d["int_vel"])
    f = torch_dev(d["int_force"])
    lib.nw_legacy_langevin_apply(ptr(f), ptr(v), ptr(noise), nb)
    with orc.force_scale(nb) as S:
        orc.langevin(cfg, d["int_force"], d["int_vel"], d["noise"], prec=64)
    S_lang = norms(d["int_force"]) + S.values[:nb]
    assert force_err(host(f), d["lang_force"], S_lang) < TOL
    # bending + tangents
    f = torch_dev(d["lang_force"])
    t = torch_dev(d["tan_in"])
    lib.filamentForces(ptr(f), ptr(t), ptr(p), float(cfg.num_filaments))
    with orc.force_scale(nb) as S:
        orc.filament(cfg, d["lang_force"], d["tan_in"], d["int_pos"], prec=64)
    S_fil = S_lang + S.values[:nb]
    assert force_err(host(f), d["fil_force"], S_fil) < TOL
    assert vec_err(host(t), d["fil_tan"]) < TOL
    # hash -> sort -> reorder: bit-exact
    import torch

    h = torch.empty(nb, dtype=torch.int32, device="cuda")
    ix = torch.empty(nb, dtype=torch.int32, device="cuda")
    lib.calcHash(ptr(h), ptr(ix), ptr(p), nb, False)
    assert np.array_equal(host(h).view(np.uint32), d["hash"])
    lib.sortParticles(ptr(h), ptr(ix), nb)
    assert np.array_equal(host(h).view(np.uint32), d["sorted_hash"])
    assert np.array_equal(host(ix).view(np.uint32), d["sorted_index"])
    ncell = cfg.n_cells
    cs = torch.empty(ncell, dtype=torch.int32, device="cuda")
    ce = torch.full((ncell,), -1, dtype=torch.int32, device="cuda")
    sp, sv, st = (torch.empty((nb, 4), dtype=torch.float32, device="cuda") for _ in range(3))
    t_in = torch_dev(d["fil_tan"])
    lib.reorderDataAndFindCellStart(ptr(cs), ptr(ce), ptr(sp), ptr(sv), ptr(st), ptr(h), ptr(ix), ptr(p), ptr(v),
                                    ptr(t_in), nb, ncell)
    csn, cen = host(cs).view(np.uint32), host(ce).view(np.uint32)
    assert np.array_equal(csn, d["cell_start"])
    ne = csn != 0xFFFFFFFF
    assert np.array_equal(cen[ne], d["cell_end"][ne])
    assert np.array_equal(host(sp), d["sorted_pos"])
    # DEM contact + cell-list bond + extensile drive
    f = torch_dev(d["fil_force"])
    # every device buffer stays referenced until the kernel has run
    bufs = [torch_dev(d["sorted_pos"]), torch_dev(d["sorted_vel"]), torch_dev(d["sorted_tan"]),
            torch_dev(d["sorted_index"].view(np.int32)), torch_dev(d["cell_start"].view(np.int32)),
            torch_dev(d["cell_end"].view(np.int32))]
    lib.collideFilaments(ptr(f), *[ptr(b) for b in bufs], nb, ncell)
    torch.cuda.synchronize()
    del bufs
    with orc.force_scale(nb) as S:
        orc.pair(cfg, d["fil_force"], d["int_pos"], d["int_vel"], d["fil_tan"], d["sorted_index"], d["cell_start"],
                 d["cell_end"], prec=64)
    assert force_err(host(f), d["collide_force"], S_fil + S.values[:nb]) < TOL
    assert lib.nw_legacy_last_status() == 0


def test_legacy_reverse_matches_reference(lib):
    cfg, d = load("ref_dem_2d.npz")
    c2 = cfg.copy()
    c2.reverse_probability = 0.3
    set_legacy_params(lib, c2)
    f, fo, v, p = (torch_dev(d[k]) for k in ("int_force", "int_force_old", "int_vel", "int_pos"))
    uni = torch_dev(d["uniform"])
    lib.nw_legacy_reverse_apply(ptr(f), ptr(fo), ptr(v), ptr(p), ptr(uni), cfg.num_filaments)
    for t, k in ((p, "rev_pos"), (v, "rev_vel"), (f, "rev_force"), (fo, "rev_force_old")):
        assert np.array_equal(host(t), d[k]), k


def test_legacy_srd_pipeline_matches_reference(lib):
    import torch

    cfg, d = load("ref_srd_2d.npz")
    set_legacy_params(lib, cfg, tuple(float(x) for x in d["shift"]))
    n = cfg.n_beads + cfg.n_solvent
    p, v = torch_dev(d["pos_in"]), torch_dev(d["vel_in"])
    h = torch.empty(n, dtype=torch.int32, device="cuda")
    ix = torch.empty(n, dtype=torch.int32, device="cuda")
    lib.calcHash(ptr(h), ptr(ix), ptr(p), n, True)
    assert np.array_equal(host(h).view(np.uint32), d["hash"])
    lib.sortParticles(ptr(h), ptr(ix), n)
    assert np.array_equal(host(ix).view(np.uint32), d["sorted_index"])
    ncell = cfg.n_cells
    nsc = cfg.n_srd_cells
    cs = torch.empty(ncell, dtype=torch.int32, device="cuda")
    ce = torch.full((ncell,), -1, dtype=torch.int32, device="cuda")
    sp, sv = (torch.empty((n, 4), dtype=torch.float32, device="cuda") for _ in range(2))
    lib.reorderDataAndFindCellStart(ptr(cs), ptr(ce), ptr(sp), ptr(sv), None, ptr(h), ptr(ix), ptr(p), ptr(v), None, n,
                                    ncell)
    csn = host(cs).view(np.uint32)[:nsc]
    assert np.array_equal(csn, d["cell_start"])
    lib.solventIsokineticThermostat(ptr(v), ptr(sv), ptr(cs), ptr(ce), ptr(ix), nsc)
    assert vec_err(host(v), d["thermo_vel"]) < TOL
    com = torch.zeros((nsc, 4), dtype=torch.float32, device="cuda")
    lib.solventCellCentorOfMomentum(ptr(com), ptr(sv), ptr(cs), ptr(ce), ptr(ix), nsc)
    assert vec_err(host(com), d["com"]) < TOL
    uni = torch_dev(d["uniform"])
    lib.nw_legacy_collide_solvent_apply(ptr(p), ptr(v), ptr(com), ptr(uni), n)
    assert vec_err(host(v), d["coll_vel"]) < TOL
    p_before = host(p)
    lib.integrateSolvent(ptr(p), ptr(v), float(d["dt_srd"]), cfg.n_beads, cfg.n_solvent)
    nb = cfg.n_beads
    assert np.array_equal(host(p)[:nb], d["pos_out"][:nb])
    assert update_err(host(p)[nb:], d["pos_out"][nb:], p_before[nb:], box_of(cfg)) < TOL
    assert vec_err(host(v), d["vel_out"]) < TOL


def test_legacy_sort_is_stable_for_arbitrary_keys(lib):
    import torch

    rng = np.random.default_rng(0)
    for n, hi in ((1, 5), (2047, 3), (2048, 1 << 32), (100003, 17), (250000, 1 << 20)):
        keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
        vals = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
        order = np.argsort(keys, kind="stable")
        k, vv = torch_dev(keys.view(np.int32)), torch_dev(vals.view(np.int32))
        lib.sortParticles(ptr(k), ptr(vv), n)
        assert np.array_equal(host(k).view(np.uint32), keys[order])
        assert np.array_equal(host(vv).view(np.uint32), vals[order])


def test_legacy_random_fills(lib):
    import torch

    lib.nw_legacy_seed(123)
    u = torch.empty(100001, dtype=torch.float32, device="cuda")
    lib.randomizeUniform(ptr(u), u.numel())
    un = host(u)
    assert un.min() > 0.0 and un.max() < 1.0 and abs(un.mean() - 0.5) < 0.01
    g = torch.empty(100003, dtype=torch.float32, device="cuda")
    lib.randomizeGaussian(ptr(g), g.numel(), 1.0, 2.0)
    gn = host(g)
    assert abs(gn.mean() - 1.0) < 0.03 and abs(gn.std() - 2.0) < 0.03
