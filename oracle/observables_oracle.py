"""numpy restatement of the observables (include/nwgb.h, "observables").

TEST INFRASTRUCTURE ONLY: the checker of nw_observe,
nw_velocity_correlation and nw_srd_temperature_histogram.

Tangents and the order parameters follow the reference's offline analysis:
analysis/afa/utils.py:35-49 (compute_tangents: windows centred on beads
1 .. n-2, one-sided at filament ends, the first and last bead of the frame
left at zero) and analysis/analyze_correlations.py:13-38
(compute_relative_orientations: Q = 1.5 t t - I/2 averaged over sampled
beads, S its largest eigenvalue, P = |mean tangent|, periodic pair
distances).  tests/golden/make_order_golden.py runs those reference
functions on seeded frames; tests/test_observables.py pins this file to them.
"""
from __future__ import annotations

import numpy as np

FIX = 4294967296.0  # 2^32, the fixed point of the SRD cell sums


def tangents(r: np.ndarray, L: int, box=None) -> np.ndarray:
    """Bead tangents (analysis/afa/utils.py:35-49) in the positions' dtype;
    with box, differences by the minimum image on the axes of positive
    length."""
    r = np.asarray(r)[:, :3]
    n = len(r)
    t = np.zeros_like(r)
    for i in range(1, n - 1):
        im1, ip1 = i - 1, i + 1
        if i % L == 0:
            im1 = i
        if i % L == L - 1:
            ip1 = i
        dr = r[ip1] - r[im1]
        if box is not None:
            dr = wrap(dr, box)
        t[i] = dr / np.linalg.norm(dr)
    return t


def wrap(d: np.ndarray, box) -> np.ndarray:
    """Minimum image in float32 as the device takes it: d - L rint(d / L)."""
    d = np.array(d, dtype=np.float32, copy=True)
    for a in range(3):
        if box[a] > 0:
            Lf = np.float32(box[a])
            d[..., a] = d[..., a] - Lf * np.rint(d[..., a] / Lf)
    return d


def relative_orientations(r: np.ndarray, t: np.ndarray, i: np.ndarray, j: np.ndarray, box):
    """compute_relative_orientations (analysis/analyze_correlations.py:13-38)
    for given sample indices: (pair distances, |t_i . t_j|, t_i . t_j, S, P)."""
    ti, tj = t[i], t[j]
    tt = np.sum(ti * tj, axis=1)
    Q = 1.5 * np.einsum("...j,...k->...jk", ti, ti)
    for a in range(3):
        Q[:, a, a] -= 0.5
    S = np.linalg.eigvalsh(Q.mean(axis=0).astype(np.float64)).max()
    P = np.linalg.norm(t.mean(axis=0))
    dr = r[i] - r[j]
    for a in range(2):
        dr[:, a][dr[:, a] > box[a] / 2] -= box[a]
        dr[:, a][dr[:, a] < -box[a] / 2] += box[a]
    return np.linalg.norm(dr, axis=1), np.abs(tt), tt, S, P


def order_parameters(t: np.ndarray) -> dict:
    """S of the mean Q over all beads (zero tangents included), S2D over the
    beads with a tangent, P = |mean tangent| over all beads (float64)."""
    t = np.asarray(t, dtype=np.float64)
    n = len(t)
    Q = 1.5 * np.einsum("ij,ik->jk", t, t) / n - 0.5 * np.eye(3)
    has = np.linalg.norm(t, axis=1) > 0
    x, y = t[has, 0], t[has, 1]
    q = x * x + y * y
    ok = q > 0
    c2 = ((x * x - y * y)[ok] / q[ok]).sum()
    s2 = ((2.0 * x * y)[ok] / q[ok]).sum()
    nt = max(int(has.sum()), 1)
    return {"s_q3": float(np.linalg.eigvalsh(Q).max()), "s_2d": float(np.hypot(c2, s2) / nt),
            "polar": float(np.linalg.norm(t.mean(axis=0))), "n_tangents": int(has.sum())}


def temperature(vel: np.ndarray, dim: int) -> float:
    v = np.asarray(vel, dtype=np.float64)
    return float((v[:, 3] * (v[:, :dim] ** 2).sum(1)).sum() / (dim * len(v))) if len(v) else 0.0


def bin_weights(d: np.ndarray, r_max: float, bins: int) -> tuple[np.ndarray, np.ndarray]:
    """Quadratic B-spline bin weights: (centre index c, weights of c-1, c, c+1)."""
    x = d / (r_max / bins) - 0.5
    c = np.floor(x + 0.5)
    t = x - c
    w = np.stack([0.5 * (0.5 - t) ** 2, 0.75 - t * t, 0.5 * (0.5 + t) ** 2], axis=-1)
    return c.astype(np.int64), w


def velocity_correlation_sums(pos, vel, i, j, box, r_max: float = 8.0, bins: int = 32):
    """(sum w v_i . v_j, sum w) per bin over the pairs (i[k], j[k]); the
    separation taken in float32 with the minimum image, its length in double."""
    p = np.asarray(pos, dtype=np.float32)[:, :3]
    v = np.asarray(vel, dtype=np.float32)[:, :3].astype(np.float64)
    d = wrap(p[j] - p[i], box).astype(np.float64)
    dist = np.sqrt((d * d).sum(1))
    c, w = bin_weights(dist, r_max, bins)
    dots = (v[i] * v[j]).sum(1)
    sd = np.zeros(bins)
    sw = np.zeros(bins)
    for q in range(3):
        b = c - 1 + q
        ok = (b >= 0) & (b < bins)
        np.add.at(sd, b[ok], w[ok, q] * dots[ok])
        np.add.at(sw, b[ok], w[ok, q])
    return sd, sw


def srd_cells(pos, grid, cell, origin, box, periodic, shift):
    """SRD cell index of each particle: shifted position relative to the box,
    wrapped on periodic axes, floor by the cell size, wrapped or clamped."""
    p = np.asarray(pos, dtype=np.float32)[:, :3]
    g = np.zeros((len(p), 3), np.int64)
    for a in range(3):
        if grid[a] == 1 and a == 2:
            continue
        x = (p[:, a] + np.float32(shift[a])) - np.float32(origin[a])
        if periodic[a]:
            x = np.where(x >= np.float32(box[a]), x - np.float32(box[a]), np.where(x < 0, x + np.float32(box[a]), x))
        k = np.floor(x / np.float32(cell[a])).astype(np.int64)
        g[:, a] = np.mod(k, grid[a]) if periodic[a] else np.clip(k, 0, grid[a] - 1)
    return (g[:, 2] * grid[1] + g[:, 1]) * grid[0] + g[:, 0]


def srd_temperature_histogram(pos, vel, grid, cell, origin, box, periodic, dim, shift, t_max, bins):
    """Counts by cell temperature sum m |v - u|^2 / (dim (n - 1)) from 2^32
    fixed-point cell sums of m, m v and m |v|^2, as the device forms them."""
    c = srd_cells(pos, grid, cell, origin, box, periodic, shift)
    v = np.asarray(vel, dtype=np.float32).astype(np.float64)
    m = v[:, 3]
    vz = v[:, 2] if dim >= 3 else np.zeros(len(v))
    fx = lambda x: np.rint(x * FIX).astype(np.int64)  # noqa: E731
    ncell = int(np.prod(grid))
    n = np.bincount(c, minlength=ncell)
    sums = []
    for x in (m, m * v[:, 0], m * v[:, 1], m * vz, m * (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + vz * vz)):
        acc = np.zeros(ncell, np.int64)
        np.add.at(acc, c, fx(x))
        sums.append(acc.astype(np.float64) / FIX)
    M, px, py, pz, ke2 = sums
    use = n >= 2
    rel = ke2[use] - (px[use] * px[use] + py[use] * py[use] + pz[use] * pz[use]) / M[use]
    T = rel / (dim * (n[use] - 1.0))
    b = np.floor(T / t_max * bins)
    k = np.where(b < 0, 0, np.where(b >= bins, bins, b)).astype(np.int64)
    out = np.bincount(k, minlength=bins + 1).astype(np.uint32)
    return np.concatenate([out, [np.uint32(use.sum())]])
