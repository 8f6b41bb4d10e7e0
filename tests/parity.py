"""Per-bead parity metrics of the floating-point arrays (FP32 step).

Every float assertion of the GPU tests compares bead by bead (particle by
particle for the solvent); none normalises by the largest value of an array.

* ``force_err``: max over beads of |f_gpu,i - f_ref,i| / S_i, where S_i is the
  bead's force scale from the FP64 oracle (``oracle.step(..., force_scale=True)``):
  the sum, over every force term acting on the bead, of the magnitudes of the
  term's parts before they cancel (both powers of a WCA pair, k (r + r0) of a
  bond, each projection of a bending triple, friction and noise).  A relative
  rounding error u in any part moves the net force by about u S_i at most, so
  this is the per-bead relative error for beads whose terms add up and the
  rounding-limited one for beads whose terms cancel (their net force can be
  1e-4 of S_i; FP32 itself then differs from FP64 by ~7e-7 S_i).
* ``vec_err``: max over beads of |a_i - b_i| / (|b_i| + floor) with the floor
  a fraction of the rms |b| (velocities, tangents).
* ``update_err``: the one-step update of stored FP32 values (positions):
  per component max(0, |a - b| - ulp(b)) / |delta_i|, delta = b - old (minimum
  image) the bead's own displacement.  At most tol means the two increments
  agree to tol of the bead's displacement, up to the final FP32 rounding of
  the stored position (one ulp of a coordinate near 1000 is 6e-5, far more
  than 1e-5 of a displacement of 1e-3).

The bar is 1e-5 against the FP32 oracle (the reference's own arithmetic in
its own order).  Against the FP64 oracle the FP32 step cannot reach 1e-5 of
the force scale on beads far from the origin: the integrator rounds positions
to FP32 (half an ulp is 3e-5 at |r| = 500), and a bond stretched by that much
changes its force by k x 3e-5.  ``fp64_bound`` therefore holds the GPU to the
FP64 error of the FP32 oracle itself: the GPU is no further from FP64 than
the reference's own FP32 computation of the same step.

Solvent velocities after an SRD collision are the cell mean plus a rotated
relative velocity.  The cell mean is a sum over the cell's members, so its
rounding scales with the members' speeds (the rms speed), not with the mean
itself, and it cancels against the rotated part for slow particles: solvent
velocities (and their streamed displacements) are compared relative to
|v| + v_rms (``SOLVENT_FLOOR`` = 1).  A cell of 215 members summed in a
different order moves a slow particle's velocity by ~1e-6 v_rms.
"""
from __future__ import annotations

import numpy as np

TOL = 1e-5
SOLVENT_FLOOR = 1.0


def fp64_bound(err_fp32_vs_fp64: float) -> float:
    """The bar against FP64: 1e-5, or 1.5 x the FP32 oracle's own FP64 error."""
    return max(TOL, 1.5 * err_fp32_vs_fp64)


def _xyz(a):
    return np.asarray(a, dtype=np.float64)[..., :3]


def force_err(a, b, scale) -> float:
    d = np.linalg.norm(_xyz(a) - _xyz(b), axis=-1)
    s = np.asarray(scale, dtype=np.float64)
    if d.size == 0:
        return 0.0
    zero = s == 0
    assert np.all(d[zero] == 0), "force on a bead with no force terms"
    return float((d[~zero] / s[~zero]).max()) if (~zero).any() else 0.0


def vec_err(a, b, floor_frac: float = 1e-3) -> float:
    a, b = _xyz(a), _xyz(b)
    if b.shape[0] == 0:
        return 0.0
    nb = np.linalg.norm(b, axis=-1)
    floor = floor_frac * (np.sqrt((nb ** 2).mean()) + 1e-300)
    return float((np.linalg.norm(a - b, axis=-1) / (nb + floor)).max())


def update_err(a, b, old, box=None, floor_frac: float = 0.0) -> float:
    a32 = np.asarray(a, dtype=np.float32)[..., :3]
    b32 = np.asarray(b, dtype=np.float32)[..., :3]
    if b32.shape[0] == 0:
        return 0.0
    delta = b32.astype(np.float64) - _xyz(old)
    if box is not None:
        L = np.asarray(box, dtype=np.float64)[:3]
        delta -= L * np.round(delta / np.where(L > 0, L, 1.0))
    dn = np.linalg.norm(delta, axis=-1)
    if floor_frac:
        dn = dn + floor_frac * np.sqrt((dn ** 2).mean())
    ulp = np.spacing(np.abs(b32)).astype(np.float64)
    excess = np.maximum(np.abs(a32.astype(np.float64) - b32.astype(np.float64)) - ulp, 0.0)
    moved = dn > 0
    assert np.all(excess[~moved] == 0), "a bead that did not move differs by more than one ulp"
    return float((excess[moved] / dn[moved, None]).max()) if moved.any() else 0.0


def summary(a, b) -> str:
    """Plain per-bead relative differences (no floor, no scale) for reports."""
    a, b = _xyz(a), _xyz(b)
    d = np.linalg.norm(a - b, axis=-1)
    nb = np.linalg.norm(b, axis=-1)
    r = d[nb > 0] / nb[nb > 0]
    if r.size == 0:
        return "empty"
    return f"max {r.max():.2e} p99.9 {np.percentile(r, 99.9):.2e} median {np.median(r):.2e}"
