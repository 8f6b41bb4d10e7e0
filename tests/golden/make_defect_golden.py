"""Generate tests/golden/defects_2d.npz: defect lists the reference's own
analysis code gives on seeded synthetic worm frames.

Runs the reference's Python functions in place (read-only checkout given by
--reference): analysis/make_director_field.py compute_director, then the
director field handed to analysis/find_defects.py compute_theta and
find_defects as read_vector_field would hand it over (the y component of the
director negated, as make_director_field.py:79 writes it), without the text
round trip; and analysis/defects.py search_for_defects, the sampling search,
on four of the frames.  The reference's code uses the ``np.int`` alias that numpy 2
removed; it is put back as ``int`` for the run.

Frames are translated so that the lowest bead sits at (1, 1) exactly: the
reference recovers cell indices from cell centres by floor((R - origin) /
cellsize), which is exact only when the centres are (as here) exactly
representable.

usage: python tests/golden/make_defect_golden.py --reference <checkout>
"""
from __future__ import annotations

import argparse
import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def worm_frame(rng, box, n_worms, L, bond, field, jitter):
    """n_worms straight worms of L beads, centres uniform in the box interior,
    each along field(centre) plus Gaussian jitter; float32 positions."""
    margin = 0.5 * (L - 1) * bond + 1.0
    c = rng.uniform(margin, box - margin, size=(n_worms, 2))
    a = field(c[:, 0], c[:, 1]) + rng.normal(0.0, jitter, n_worms)
    k = np.arange(L) - 0.5 * (L - 1)
    x = c[:, None, 0] + bond * k[None, :] * np.cos(a)[:, None]
    y = c[:, None, 1] + bond * k[None, :] * np.sin(a)[:, None]
    r = np.stack([x.ravel(), y.ravel()], 1)
    r = r - r.min(axis=0) + 1.0  # lowest bead at (1, 1)
    out = np.zeros((len(r), 3), dtype=np.float32)
    out[:, :2] = r.astype(np.float32)
    return out


def planted(defects):
    """Director angle field of point defects [(x, y, charge), ...]."""
    def f(x, y):
        return sum(q * np.arctan2(y - y0, x - x0) for x0, y0, q in defects)
    return f


def lattice_frame(L):
    """Worms on a lattice: horizontal rows in the lower half, vertical columns
    in the upper right, an empty upper-left block; exact 0 and pi/2 director
    angles next to empty cells."""
    rows = []
    for j in range(0, 20, 2):
        for i in range(0, 40, L + 1):
            rows.append([(i + k, j) for k in range(L)])
    for i in range(20, 40, 2):
        for j in range(22, 40, L + 1):
            rows.append([(i, j + k) for k in range(L)])
    r = np.array(rows, dtype=np.float64).reshape(-1, 2) + 1.0
    out = np.zeros((len(r), 3), dtype=np.float32)
    out[:, :2] = r
    return out


def diagonal_frame(L):
    """Worms at exactly +45 and -45 degrees beside horizontal ones and an
    empty block: director angles of exactly -pi/4, pi/4 and 0 side by side."""
    rows = []
    for j in range(0, 16, 2):
        for i in range(0, 36, L + 1):
            rows.append([(i + k, j) for k in range(L)])
    for s in range(0, 30, 3):
        rows.append([(s + k, 18 + k) for k in range(L)])        # +45
        rows.append([(s + k, 36 - k) for k in range(L)])        # -45
    r = np.array(rows, dtype=np.float64).reshape(-1, 2) + 1.0
    out = np.zeros((len(r), 3), dtype=np.float32)
    out[:, :2] = r
    return out


def pinwheel_frame(L):
    """Four lattice quadrants, horizontal and vertical worms alternating round
    the centre: neighbouring director angles differ by exactly pi/2, where the
    circuit's step reduction depends on the angles' representatives."""
    rows = []
    for qx in range(2):
        for qy in range(2):
            x0, y0 = 24 * qx, 24 * qy
            if (qx + qy) % 2 == 0:
                for j in range(0, 24, 2):
                    for i in range(0, 24 - L, L + 1):
                        rows.append([(x0 + i + k, y0 + j) for k in range(L)])
            else:
                for i in range(0, 24, 2):
                    for j in range(0, 24 - L, L + 1):
                        rows.append([(x0 + i, y0 + j + k) for k in range(L)])
    r = np.array(rows, dtype=np.float64).reshape(-1, 2) + 1.0
    out = np.zeros((len(r), 3), dtype=np.float32)
    out[:, :2] = r
    return out


def junction_frame(L):
    """Horizontal worms lower left, vertical lower right, +45 degree worms in
    the upper half: rings round the junction step horizontal -> vertical ->
    diagonal, whose total depends on the vertical director's representative
    (-pi/2 from the reference's eigen-solver)."""
    rows = []
    for j in range(0, 24, 2):
        for i in range(0, 24 - L, L + 1):
            rows.append([(i + k, j) for k in range(L)])
    for i in range(24, 48, 2):
        for j in range(0, 24 - L, L + 1):
            rows.append([(i, j + k) for k in range(L)])
    for j in range(24, 48 - L, 3):
        for i in range(0, 48 - L, 3):
            rows.append([(i + k, j + k) for k in range(L)])
    r = np.array(rows, dtype=np.float64).reshape(-1, 2) + 1.0
    out = np.zeros((len(r), 3), dtype=np.float32)
    out[:, :2] = r
    return out


def reference_defects(ref_analysis: Path, pos: np.ndarray, L: int, cellsize: float):
    sys.path.insert(0, str(ref_analysis))
    np.int = int  # removed alias used by the reference
    from afa.data import Frame
    from find_defects import compute_theta, find_defects
    from make_director_field import compute_director

    r = pos.astype(np.float64)
    frame = Frame(positions=r, labels=np.zeros(len(r)), filament_length=L)
    field = compute_director(frame, cellsize)
    R = field[:, 0:3]
    V = field[:, 3:6].copy()
    V[:, 1] = -V[:, 1]
    origin = R.min(axis=0)
    f = {"index": 1, "num_sites": len(R), "positions": R, "director": V, "origin": origin,
         "box_size": R.max(axis=0) - origin}
    f = compute_theta(f, cellsize)
    # every cell centre must map back to its own cell
    cells = np.floor((R - origin) / cellsize).astype(np.int64)
    shape = f["theta"].shape
    assert len(np.unique(cells[:, 0] * shape[1] + cells[:, 1])) == len(R), "cell centres collide"
    out = find_defects(f)
    return np.array([(x, y, q) for (_, x, y, _, q) in out], dtype=np.float64).reshape(-1, 3)


def reference_sampling(ref_analysis: Path, pos: np.ndarray, L: int, n_points: int, radius: float, seed: int):
    """The reference's sampling search, analysis/defects.py search_for_defects,
    called as its __main__ does (neighbour tree and tangents built first) with
    numpy's global generator seeded; the sample bead indices are the draw it
    makes (afa/data.py sample_points), repeated from the same seed.  Returns the
    indices and the kept points' values (winding > 0) in draw order."""
    sys.path.insert(0, str(ref_analysis))
    from afa.data import Frame
    from defects import search_for_defects

    r = pos.astype(np.float64)
    frame = Frame(positions=r, labels=np.zeros(len(r)), filament_length=L)
    frame.build_neighbors_list()
    frame.compute_filament_tangents()
    np.random.seed(seed)
    dc = search_for_defects(frame, {"radius": radius, "n_points": n_points})
    np.random.seed(seed)
    beads = np.random.randint(0, len(frame), size=n_points).astype(np.uint32)
    kept = np.array([[p[0], p[1], v] for p, v in zip(dc.r, dc.v)], dtype=np.float64).reshape(-1, 3)
    return beads, kept


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="checkout of the reference project")
    args = ap.parse_args()
    ana = Path(args.reference) / "analysis"
    rng = np.random.default_rng(20261203)
    cases = {
        "pair_c2": (worm_frame(rng, 64.0, 900, 5, 0.8, planted([(20, 32, 0.5), (44, 32, -0.5)]), 0.1), 5, 2.0),
        "quad_c3": (worm_frame(rng, 96.0, 2400, 6, 0.7,
                               planted([(24, 24, 0.5), (72, 24, -0.5), (24, 72, -0.5), (72, 72, 0.5)]), 0.15), 6, 3.0),
        "nematic_c2": (worm_frame(rng, 48.0, 500, 8, 0.8, lambda x, y: 0.3 + 0 * x, 0.05), 8, 2.0),
        "isotropic_c2": (worm_frame(rng, 40.0, 400, 4, 0.8, lambda x, y: 0 * x, math.pi), 4, 2.0),
        "lattice_c2": (lattice_frame(5), 5, 2.0),
        "diagonal_c2": (diagonal_frame(5), 5, 2.0),
        "pinwheel_c2": (pinwheel_frame(5), 5, 2.0),
        "junction_c2": (junction_frame(5), 5, 2.0),
    }
    arrays = {}
    for name, (pos, L, cs) in cases.items():
        d = reference_defects(ana, pos, L, cs)
        arrays[f"{name}_pos"] = pos[:, :2]
        arrays[f"{name}_meta"] = np.array([L, cs])
        arrays[f"{name}_defects"] = d
        print(f"{name}: {len(pos)} beads, L={L}, cellsize={cs}: {len(d)} defects "
              f"(+{int((d[:, 2] > 0).sum())} / -{int((d[:, 2] < 0).sum())})")
        if name in ("pair_c2", "quad_c3", "isotropic_c2", "junction_c2"):
            beads, kept = reference_sampling(ana, pos, L, 200, 6.0, seed=len(pos))
            arrays[f"{name}_sample_beads"] = beads
            arrays[f"{name}_sample_kept"] = kept
            print(f"  sampling search: 200 points, radius 6: {len(kept)} kept")
    np.savez_compressed(HERE / "defects_2d.npz", **arrays)


if __name__ == "__main__":
    main()
