"""Device defect finder (nw_find_defects) against the reference's defect lists
(tests/golden/defects_2d.npz) and against the defect oracle
(oracle/defects_oracle.py) on larger frames and on simulated states: the
same defects, positions bit-identical."""
from __future__ import annotations

import numpy as np
import pytest

import defects_oracle as D
from conftest import GOLDEN as GOLDEN_DIR
from nwgb import abi
from nwgb.init import initial_state, wca_config

pytestmark = pytest.mark.gpu

GOLDEN = np.load(GOLDEN_DIR / "defects_2d.npz")
NAMES = sorted(k[:-4] for k in GOLDEN.files if k.endswith("_pos"))


def rows(d):
    return np.stack([d["x"], d["y"], d["charge"].astype(np.float64)], 1) if len(d) else np.zeros((0, 3))


def system_with(lib, pos2, L, box=None):
    import nwgb

    n = len(pos2)
    box = box or (float(np.ceil(pos2[:, 0].max() + 2)), float(np.ceil(pos2[:, 1].max() + 2)))
    cfg = wca_config(n // L, L, box, lib=lib)
    s = nwgb.System(cfg)
    p = np.zeros((n, 4), dtype=np.float32)
    p[:, :2] = pos2
    s.set_array(abi.NW_POSITION, p)
    return s


@pytest.mark.parametrize("name", NAMES)
def test_device_defects_match_reference(lib, name):
    pos = GOLDEN[name + "_pos"]
    L, cs = GOLDEN[name + "_meta"]
    with system_with(lib, pos, int(L)) as s:
        got = s.find_defects(float(cs))
    want = GOLDEN[name + "_defects"]
    assert rows(got).shape == want.shape
    assert np.array_equal(rows(got), want)


def planted_frame(rng, n_worms, L, box, sites, jitter=0.1, bond=0.8):
    m = 0.5 * (L - 1) * bond + 1.0
    c = rng.uniform(m, box - m, (n_worms, 2))
    a = sum(q * np.arctan2(c[:, 1] - y, c[:, 0] - x) for x, y, q in sites) + rng.normal(0, jitter, n_worms)
    k = np.arange(L) - 0.5 * (L - 1)
    return np.stack([(c[:, None, 0] + bond * k * np.cos(a)[:, None]).ravel(),
                     (c[:, None, 1] + bond * k * np.sin(a)[:, None]).ravel()], 1).astype(np.float32)


@pytest.mark.parametrize("n_worms,L,box,cs", [(20000, 10, 400.0, 2.0), (40000, 5, 300.0, 1.5), (100000, 4, 1000.0, 4.0)])
def test_device_defects_match_oracle_on_large_frames(lib, n_worms, L, box, cs):
    rng = np.random.default_rng(n_worms + L)
    sites = [(rng.uniform(0.2, 0.8) * box, rng.uniform(0.2, 0.8) * box, q) for q in (0.5, -0.5, 0.5, -0.5)]
    pos = planted_frame(rng, n_worms, L, box, sites, jitter=0.3)
    with system_with(lib, pos, L) as s:
        got = s.find_defects(cs)
    want = D.find_defects(pos, L, cs)
    assert len(want) > 4
    assert np.array_equal(rows(got), rows(want))
    assert np.array_equal(got["cells"], want["cells"])


def test_min_image_tangents_through_the_boundary(lib):
    """Worms wrapped through the periodic boundary: with NW_DEFECT_MIN_IMAGE the
    tangents are the physical ones; without it the raw differences (the
    reference's) are taken."""
    rng = np.random.default_rng(5)
    box = 60.0
    # a +1/2, -1/2 pair one above the other, moved against the x edge: the
    # worms round the pair straddle the periodic boundary
    pos = planted_frame(rng, 4000, 6, box, [(30, 20, 0.5), (30, 40, -0.5)], jitter=0.05)
    pos[:, 0] = (pos[:, 0] + np.float32(29.0)) % np.float32(box)
    with system_with(lib, pos, 6, box=(box, box)) as s:
        raw = s.find_defects(2.0)
        img = s.find_defects(2.0, min_image=True)
    assert np.array_equal(rows(raw), rows(D.find_defects(pos, 6, 2.0)))
    assert np.array_equal(rows(img), rows(D.find_defects(pos, 6, 2.0, box=(box, box))))
    assert not np.array_equal(rows(raw), rows(img))


@pytest.mark.parametrize("strategy", [abi.NW_STRATEGY_SORTED, abi.NW_STRATEGY_CELL_LISTS, abi.NW_STRATEGY_VERLET])
def test_device_defects_of_a_simulated_state(lib, strategy):
    """After stepping (odd step count: the current state sits in the second
    buffer of the double-buffered strategies) the finder reads the state the
    system reports."""
    import nwgb

    cfg = wca_config(300, 10, (100.0, 100.0), seed=9, lib=lib)
    cfg.strategy = strategy
    pos, vel = initial_state(cfg, seed=9)
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.step(301, cfg.dt)
        got = s.find_defects(2.0, min_image=True)
        p = s.get_array(abi.NW_POSITION)[: cfg.n_beads]
    want = D.find_defects(p[:, :2], cfg.filament_size, 2.0, box=(cfg.box[0], cfg.box[1]))
    assert np.array_equal(rows(got), rows(want))
    assert np.array_equal(got["cells"], want["cells"])


def test_defect_finder_argument_checks(lib):
    import nwgb

    cfg = wca_config(4, 5, (10.0, 10.0), lib=lib)
    with nwgb.System(cfg) as s:
        for bad in (0.0, -1.0, float("nan"), float("inf")):
            with pytest.raises(nwgb.NwError) as e:
                s.find_defects(bad)
            assert e.value.status == abi.NW_ERR_INVALID


def test_defect_finder_edge_cases(lib):
    """A frame too small for an interior cell has no defects; a short output
    buffer still reports the full count; non-finite positions are refused;
    3D systems are not supported."""
    import ctypes as C

    import nwgb

    with system_with(lib, GOLDEN["pair_c2_pos"][:10], 5) as s:  # two worms: a 3 x 2 grid at most
        assert len(s.find_defects(2.0)) == 0
    pos = GOLDEN["isotropic_c2_pos"]
    want = D.find_defects(pos, 4, 2.0)
    with system_with(lib, pos, 4) as s:
        buf = (abi.NwDefect * 1)()
        n = C.c_int()
        abi.check(lib.nw_find_defects(s._h, C.c_float(2.0), 0, buf, 1, C.byref(n)))
        assert n.value == len(want) > 1
        assert (buf[0].x, buf[0].y, buf[0].charge) == (want["x"][0], want["y"][0], want["charge"][0])
        assert np.array_equal(rows(s.find_defects(2.0, max_defects=2)), rows(want))  # grows its buffer
        p = s.get_array(abi.NW_POSITION)
        p[7, 0] = np.nan
        s.set_array(abi.NW_POSITION, p)
        with pytest.raises(nwgb.NwError) as e:
            s.find_defects(2.0)
        assert e.value.status == abi.NW_ERR_INVALID
    cfg3 = abi.default_config(abi.NW_MODEL_WCA_WORMS, 16, 10, (12, 12, 12), False, lib)
    with nwgb.System(cfg3) as s:
        with pytest.raises(nwgb.NwError) as e:
            s.find_defects(2.0)
        assert e.value.status == abi.NW_ERR_UNSUPPORTED


SAMPLED = sorted(k[: -len("_sample_beads")] for k in GOLDEN.files if k.endswith("_sample_beads"))


@pytest.mark.parametrize("name", SAMPLED)
def test_device_sampling_search_matches_reference(lib, name):
    pos = GOLDEN[name + "_pos"]
    L, _ = GOLDEN[name + "_meta"]
    beads = GOLDEN[name + "_sample_beads"]
    with system_with(lib, pos, int(L)) as s:
        w = s.sample_defects(beads, 6.0)
    assert np.array_equal(w, D.sample_windings(pos, int(L), beads, 6.0))
    sel = w > 0
    got = np.stack([pos[beads[sel], 0].astype(np.float64), pos[beads[sel], 1].astype(np.float64),
                    w[sel].astype(np.float64)], 1)
    assert np.array_equal(got, GOLDEN[name + "_sample_kept"])


def test_device_sampling_search_on_a_large_frame(lib):
    rng = np.random.default_rng(12)
    pos = planted_frame(rng, 20000, 10, 400.0, [(120, 200, 0.5), (280, 200, -0.5)], jitter=0.4)
    beads = rng.integers(0, len(pos), 300)
    with system_with(lib, pos, 10) as s:
        w = s.sample_defects(beads, 10.0)
        with pytest.raises(Exception):
            s.sample_defects([len(pos)], 10.0)  # bead index out of range
    want = D.sample_windings(pos, 10, beads, 10.0)
    assert (want != 0).any()
    assert np.array_equal(w, want)
