"""numpy restatement of the reference's defect analysis: the director field of
analysis/make_director_field.py:10-47 followed by the Burgers-circuit defect
search of analysis/find_defects.py:43-207.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the device
defect finder (nw_find_defects).  Pinned against defect lists the reference's
own Python functions produce on the frames in tests/golden/defects_2d.npz
(tests/golden/make_defect_golden.py).

The reference computes a cell's director as an eigenvector of the 3x3 tensor
Q = sum(3 t t - I) / 2N and reads its angle back as atan2(-v_y, v_x) from the
written field (make_director_field.py:42-46, 79).  In the plane the largest
eigenvector's angle is 0.5 * atan2(sum sin 2a, sum cos 2a); the eigen-solver
returns it in [-pi/4, 3pi/4), except for a diagonal tensor (sum sin 2a == 0),
where the vectors are the axes: 0 when Q_xx >= Q_yy, -pi/2 otherwise.  Empty
cells have the zero director, angle 0.  The representative matters only when
two neighbouring angles differ by exactly pi/2, which the step reduction of
theta_diff breaks one way or the other.
"""
from __future__ import annotations

import math

import numpy as np

LOOP_B = [(1, 0), (1, 1), (0, 1), (-1, 1), (-1, 0), (-1, -1), (0, -1), (1, -1), (1, 0)]
DELTA = math.pi / 16


def tangents(pos: np.ndarray, filament_length: int, box=None) -> np.ndarray:
    """Unit bead tangents r[i+1] - r[i-1], one-sided at filament ends; beads 0
    and n-1 keep the zero tangent (analysis/afa/utils.py:35-49, whose windows
    are centred on beads 1 .. n-2).  With ``box`` (periodic lengths x, y) the
    differences take the single-shift minimum image of the engine's
    lengthPeriodic (particles_kernel_impl.cuh:279-301), in float32."""
    r = np.asarray(pos, dtype=np.float64)[:, :2]
    n = len(r)
    t = np.zeros((n, 2))
    if n < 3:
        return t
    i = np.arange(1, n - 1)
    c = i % filament_length
    a = np.where(c == 0, i, i - 1)
    b = np.where(c == filament_length - 1, i, i + 1)
    if box is None:
        d = r[b] - r[a]
    else:
        # the device forms the difference in float32, as the positions are
        p32 = np.asarray(pos, dtype=np.float32)[:, :2]
        d32 = p32[b] - p32[a]
        L = np.asarray(box, dtype=np.float32)[:2]
        h = L / np.float32(2.0)
        d32 = np.where(d32 > h, d32 - L, np.where(d32 < -h, d32 + L, d32))
        d = d32.astype(np.float64)
    norm = np.linalg.norm(d, axis=1)
    ok = norm > 0
    t[i[ok]] = d[ok] / norm[ok, None]
    return t


def director_angles(pos: np.ndarray, filament_length: int, cell_size: float, box=None):
    """(theta[nx, ny], origin[2]) of the director field
    (analysis/make_director_field.py:10-47, find_defects.py:43-58)."""
    r = np.asarray(pos, dtype=np.float64)[:, :2]
    origin = r.min(axis=0)
    shape = np.ceil((r.max(axis=0) - origin + 0.0001) / cell_size).astype(np.int64)
    t = tangents(pos, filament_length, box)
    cell = np.floor((r - origin) / cell_size).astype(np.int64)
    flat = cell[:, 0] * shape[1] + cell[:, 1]
    ncell = int(shape[0] * shape[1])
    C = np.bincount(flat, weights=t[:, 0] ** 2 - t[:, 1] ** 2, minlength=ncell)
    S = np.bincount(flat, weights=2.0 * t[:, 0] * t[:, 1], minlength=ncell)
    theta = 0.5 * np.arctan2(S, C)
    theta = np.where(theta < -math.pi / 4, theta + math.pi, theta)
    theta = np.where(S == 0.0, np.where(C < 0.0, -math.pi / 2, 0.0), theta)
    return theta.reshape(int(shape[0]), int(shape[1])), origin


def _step(t1, t2):
    """theta_diff (analysis/find_defects.py:62-68), elementwise."""
    d = t2 - t1
    return np.where(d >= math.pi / 2, d - math.pi, np.where(d <= -math.pi / 2, d + math.pi, d))


def circuits(theta: np.ndarray) -> np.ndarray:
    """Total director rotation along LOOP_B around every interior cell
    (analysis/find_defects.py:70-78, 170-183); 0 on the border."""
    nx, ny = theta.shape
    total = np.zeros_like(theta)
    if nx < 3 or ny < 3:
        return total
    acc = np.zeros((nx - 2, ny - 2))
    sl = lambda dx, dy: theta[1 + dx:nx - 1 + dx, 1 + dy:ny - 1 + dy]  # noqa: E731
    t1 = sl(*LOOP_B[0])
    for dx, dy in LOOP_B[1:]:
        t2 = sl(dx, dy)
        acc = acc + _step(t1, t2)
        t1 = t2
    total[1:-1, 1:-1] = acc
    return total


def _cluster(mask: np.ndarray):
    """Touching marked cells merged (8-neighbourhood, no wrap), clusters in
    order of their first cell, each as (mean i, mean j, count)
    (analysis/find_defects.py:126-160)."""
    I, J = np.nonzero(mask)
    n = len(I)
    index = {(int(i), int(j)): k for k, (i, j) in enumerate(zip(I, J))}
    parent = list(range(n))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for k, (i, j) in enumerate(zip(I, J)):
        for di, dj in LOOP_B[1:]:
            q = index.get((int(i) + di, int(j) + dj))
            if q is not None:
                ra, rb = find(k), find(q)
                if ra != rb:
                    parent[max(ra, rb)] = min(ra, rb)
    groups = {}
    for k in range(n):
        groups.setdefault(find(k), []).append(k)
    return [(float(np.mean(I[g])), float(np.mean(J[g])), len(g)) for _, g in sorted(groups.items())]


def find_defects(pos: np.ndarray, filament_length: int, cell_size: float = 2.0, box=None) -> np.ndarray:
    """Defects of a 2D frame as a structured array (x, y, charge, cells):
    positive first, each sign in order of its first cell
    (analysis/find_defects.py:163-207)."""
    theta, origin = director_angles(pos, filament_length, cell_size, box)
    total = circuits(theta)
    marked = (total > math.pi - DELTA) | (total < -math.pi + DELTA)
    centre = origin + 0.0 + cell_size / 2.0  # the first cell's centre
    rows = []
    for sign, charge in ((1, 0.5), (-1, -0.5)):
        for ci, cj, cnt in _cluster(marked & (np.sign(total) == sign)):
            rows.append((ci * cell_size + centre[0], cj * cell_size + centre[1], charge, cnt))
    return np.array(rows, dtype=[("x", "f8"), ("y", "f8"), ("charge", "f4"), ("cells", "u4")])


def sample_windings(pos: np.ndarray, filament_length: int, beads, radius: float = 10.0, box=None) -> np.ndarray:
    """Winding value around each sample bead's position, the sampling search of
    analysis/defects.py:12-32 (with analysis/afa/utils.py:4-17, 35-54): beads
    within `radius` (Euclidean, the centre included) binned into 8 sectors of
    pi/4 from -pi by np.digitize of their displacement angle, a sector's
    director the angle of its mean tangent, then round(sum(diff(angles / pi)))
    over sectors 0 .. the highest occupied (empty sectors read 0)."""
    r = np.asarray(pos, dtype=np.float64)[:, :2]
    t = tangents(pos, filament_length, box)
    edges = [(i - 4) * (2 * np.pi / 8) for i in range(8)]
    out = np.zeros(len(beads), dtype=np.int32)
    for k, b in enumerate(np.asarray(beads)):
        d = r - r[b]
        near = np.nonzero(d[:, 0] ** 2 + d[:, 1] ** 2 <= radius * radius)[0]
        sector = np.digitize(np.arctan2(d[near, 1], d[near, 0]), edges) - 1
        ids = np.unique(sector)
        angles = np.zeros(ids.max() + 1)
        for s_ in ids:
            m = t[near[sector == s_]].mean(axis=0)
            angles[s_] = np.arctan2(m[1], m[0])
        out[k] = round(np.sum(np.diff(angles / np.pi)))
    return out

