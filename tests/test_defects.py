"""The defect oracle (oracle/defects_oracle.py) against defect lists the reference's
own analysis code produced (tests/golden/defects_2d.npz, made by
tests/golden/make_defect_golden.py from analysis/make_director_field.py and
analysis/find_defects.py): bit-identical positions and charges."""
from __future__ import annotations

import math

import numpy as np
import pytest

import defects_oracle as D

from conftest import GOLDEN as GOLDEN_DIR

GOLDEN = np.load(GOLDEN_DIR / "defects_2d.npz")
NAMES = sorted(k[:-4] for k in GOLDEN.files if k.endswith("_pos"))


def as_rows(d):
    return np.stack([d["x"], d["y"], d["charge"].astype(np.float64)], 1) if len(d) else np.zeros((0, 3))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_defects(name):
    pos = GOLDEN[name + "_pos"]
    L, cs = GOLDEN[name + "_meta"]
    want = GOLDEN[name + "_defects"]
    got = as_rows(D.find_defects(pos, int(L), float(cs)))
    assert got.shape == want.shape
    assert np.array_equal(got, want)


def test_golden_frames_cover_both_signs_and_none():
    counts = {n: GOLDEN[n + "_defects"] for n in NAMES}
    assert any((d[:, 2] > 0).any() and (d[:, 2] < 0).any() for d in counts.values())
    assert any(len(d) == 0 for d in counts.values())


def test_junction_frame_tells_director_representatives_apart(monkeypatch):
    """With the plain representative (-pi/2, pi/2] instead of the reference
    eigen-solver's, the junction frame's horizontal -> vertical -> diagonal
    rings count defects the reference does not: the golden frames pin the
    representative rule, not only the defect search."""
    def plain(pos, L, cs, box=None):
        r = np.asarray(pos, dtype=np.float64)[:, :2]
        origin = r.min(0)
        shape = np.ceil((r.max(0) - origin + 1e-4) / cs).astype(np.int64)
        t = D.tangents(pos, L, box)
        cell = np.floor((r - origin) / cs).astype(np.int64)
        flat = cell[:, 0] * shape[1] + cell[:, 1]
        C = np.bincount(flat, t[:, 0] ** 2 - t[:, 1] ** 2, minlength=int(shape.prod()))
        S = np.bincount(flat, 2 * t[:, 0] * t[:, 1], minlength=int(shape.prod()))
        return (0.5 * np.arctan2(S, C)).reshape(int(shape[0]), int(shape[1])), origin

    monkeypatch.setattr(D, "director_angles", plain)
    pos = GOLDEN["junction_c2_pos"]
    L, cs = GOLDEN["junction_c2_meta"]
    assert len(D.find_defects(pos, int(L), float(cs))) != len(GOLDEN["junction_c2_defects"])


def test_planted_defect_pair_is_found_near_its_sites():
    rng = np.random.default_rng(5)
    n, L, b = 3000, 5, 0.8
    c = rng.uniform(4, 76, (n, 2))
    a = 0.5 * np.arctan2(c[:, 1] - 40, c[:, 0] - 25) - 0.5 * np.arctan2(c[:, 1] - 40, c[:, 0] - 55)
    k = np.arange(L) - 2.0
    pos = np.stack([(c[:, None, 0] + b * k * np.cos(a)[:, None]).ravel(),
                    (c[:, None, 1] + b * k * np.sin(a)[:, None]).ravel()], 1).astype(np.float32)
    d = D.find_defects(pos, L, 2.0)
    pos_def = d[d["charge"] > 0]
    neg_def = d[d["charge"] < 0]
    assert min(math.hypot(x - 25, y - 40) for x, y in zip(pos_def["x"], pos_def["y"])) < 3.0
    assert min(math.hypot(x - 55, y - 40) for x, y in zip(neg_def["x"], neg_def["y"])) < 3.0


def test_tangents_follow_the_reference_window():
    pos = np.array([[0, 0], [1, 0], [2, 0], [2, 1], [2, 2], [2, 3]], dtype=np.float32)
    t = D.tangents(pos, 3)
    assert np.all(t[0] == 0) and np.all(t[-1] == 0)  # no window is centred on the first or last bead
    assert np.allclose(t[1], [1, 0]) and np.allclose(t[2], [1, 0])  # one-sided at the filament tail
    assert np.allclose(t[3], [0, 1]) and np.allclose(t[4], [0, 1])


SAMPLED = sorted(k[: -len("_sample_beads")] for k in GOLDEN.files if k.endswith("_sample_beads"))


@pytest.mark.parametrize("name", SAMPLED)
def test_sampling_oracle_matches_reference(name):
    """The sampling search (analysis/defects.py search_for_defects, run by the
    golden script with its draw seeded): the same kept points and values."""
    pos = GOLDEN[name + "_pos"]
    L, _ = GOLDEN[name + "_meta"]
    beads = GOLDEN[name + "_sample_beads"]
    kept = GOLDEN[name + "_sample_kept"]
    w = D.sample_windings(pos, int(L), beads, 6.0)
    sel = w > 0
    got = np.stack([pos[beads[sel], 0].astype(np.float64), pos[beads[sel], 1].astype(np.float64),
                    w[sel].astype(np.float64)], 1)
    assert np.array_equal(got, kept)


def test_sampling_golden_frames_keep_points():
    assert sum(len(GOLDEN[n + "_sample_kept"]) for n in SAMPLED) > 20


@pytest.mark.parametrize("shift", [(2.0, 0.0), (-6.0, 10.0), (0.5, 0.25)])
def test_defects_follow_a_translated_frame(shift):
    """The grid starts at the beads' own lowest corner, so a frame moved by an
    exact offset (in float64, as the analysis reads positions) keeps its
    cells: the same defects, moved by the offset."""
    pos = GOLDEN["pair_c2_pos"].astype(np.float64)
    moved = pos + np.array(shift)
    a = D.find_defects(pos, 5, 2.0)
    b = D.find_defects(moved, 5, 2.0)
    assert len(a) == len(b) > 0
    assert np.array_equal(a["charge"], b["charge"]) and np.array_equal(a["cells"], b["cells"])
    assert np.allclose(b["x"] - a["x"], shift[0], atol=1e-9) and np.allclose(b["y"] - a["y"], shift[1], atol=1e-9)
