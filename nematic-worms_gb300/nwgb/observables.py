"""Observables of a worm state as differentiable torch functions: bead
tangents, nematic order, velocity correlation by distance, kinetic
temperature, mean-square displacement, and the loss the adjoint rollout is
checked with.  Positions and velocities are (n_replicas, n_beads, 3) tensors
(float4 arrays reshape to that with as_rn3); every function works per
replica.

Definitions follow the reference's analysis code where it has one:
tangents t_i = unit(r_{i+1} - r_{i-1}), one-sided at the filament ends
(analysis/afa/utils.py:35-49, here with the minimum image); the nematic
order from the 3D Q tensor Q = 1.5 <t t> - I/2
(analysis/analyze_correlations.py:22-28), whose largest eigenvalue for
planar tangents is 1/4 + 3/4 S2 with S2 = |<exp(2 i theta)>|; the loss uses
S2.  The velocity correlation C_v(r) (mean v_i . v_j of sampled bead pairs
at distance r, normalised by <|v|^2>, with smooth bin weights) has no
reference definition and is defined here.
"""
from __future__ import annotations

import torch


def min_image(d: torch.Tensor, box: torch.Tensor) -> torch.Tensor:
    """Single-shift minimum image: d -/+ box where |d| > box / 2."""
    half = box / 2
    return torch.where(d > half, d - box, torch.where(d < -half, d + box, d))


def bead_tangents(pos: torch.Tensor, L: int, box) -> torch.Tensor:
    """Unit tangents (R, nb, 3); pos (R, nb, 3) with nb a multiple of L."""
    box = torch.as_tensor(box, dtype=pos.dtype, device=pos.device)
    R, nb, _ = pos.shape
    r = pos.reshape(R, nb // L, L, 3)
    nxt = torch.cat([r[:, :, 1:], r[:, :, -1:]], dim=2)
    prv = torch.cat([r[:, :, :1], r[:, :, :-1]], dim=2)
    d = min_image(nxt - prv, box)
    t = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    return t.reshape(R, nb, 3)


def nematic_s2(t: torch.Tensor) -> torch.Tensor:
    """2D nematic order |<exp(2 i theta)>| per replica, t (R, nb, 3) unit."""
    c = (t[..., 0] ** 2 - t[..., 1] ** 2).mean(dim=1)
    s = (2.0 * t[..., 0] * t[..., 1]).mean(dim=1)
    return torch.sqrt(c * c + s * s)


def nematic_q3(t: torch.Tensor) -> torch.Tensor:
    """Largest eigenvalue of the mean 3D Q tensor 1.5 <t t> - I/2 per replica."""
    Q = 1.5 * torch.einsum("rni,rnj->rij", t, t) / t.shape[1]
    Q = Q - 0.5 * torch.eye(3, dtype=t.dtype, device=t.device)
    return torch.linalg.eigvalsh(Q)[:, -1]


def polar_order(t: torch.Tensor) -> torch.Tensor:
    """|<t>| per replica."""
    return torch.linalg.norm(t.mean(dim=1), dim=-1)


def kinetic_temperature(vel: torch.Tensor, dim: int = 2, mass: float = 1.0) -> torch.Tensor:
    """<m |v|^2> / dim per replica."""
    return mass * (vel[..., :dim] ** 2).sum(-1).mean(dim=1) / dim


def mean_square_displacement(unwrapped: torch.Tensor, ref: torch.Tensor) -> torch.Tensor:
    """<|r - r_ref|^2> of unwrapped positions per replica."""
    return ((unwrapped - ref) ** 2).sum(-1).mean(dim=1)


class PairSample:
    """Fixed random bead pairs per replica (the reference's analysis samples
    pairs the same way) for the velocity correlation."""

    def __init__(self, n_replicas: int, n_beads: int, n_pairs: int, seed: int = 0, device="cpu"):
        g = torch.Generator().manual_seed(seed)
        i = torch.randint(0, n_beads, (n_replicas, n_pairs), generator=g)
        j = torch.randint(0, n_beads - 1, (n_replicas, n_pairs), generator=g)
        j = j + (j >= i).long()  # never i itself
        self.i, self.j = i.to(device), j.to(device)


def bin_weights(d: torch.Tensor, r_max: float, bins: int) -> torch.Tensor:
    """Weights (..., bins) of distances d on `bins` bins of width r_max / bins
    by the quadratic B-spline around the bin centres: each distance spreads
    over its nearest centre and the two beside it with weights summing to 1
    (weight beyond the first or last bin is dropped).  The weights, and
    every average built from them, are continuously differentiable in d, so
    the loss below has the gradient its adjoint computes; hard bin membership
    would make it jump wherever a pair crosses a bin edge."""
    x = d / (r_max / bins) - 0.5
    c = torch.floor(x + 0.5)
    t = x - c
    w = torch.stack([0.5 * (0.5 - t) ** 2, 0.75 - t * t, 0.5 * (0.5 + t) ** 2], dim=-1)
    idx = c.long()[..., None] + torch.tensor([-1, 0, 1], device=d.device)
    ok = (idx >= 0) & (idx < bins)
    out = torch.zeros(d.shape + (bins + 1,), dtype=d.dtype, device=d.device)
    out.scatter_add_(-1, torch.where(ok, idx, torch.full_like(idx, bins)), torch.where(ok, w, torch.zeros_like(w)))
    return out[..., :bins]


def velocity_correlation(pos: torch.Tensor, vel: torch.Tensor, pairs: PairSample, box, r_max: float = 8.0,
                         bins: int = 32) -> torch.Tensor:
    """C_v per replica and distance bin (R, bins): the mean of v_i . v_j over
    the sampled pairs, each weighted into the bins of its (minimum-image)
    distance by bin_weights, divided by <|v|^2>.  A bin's mean is its weighted
    sum over its weight sum plus 1e-3 (so that nearly empty bins stay finite
    and smooth)."""
    box = torch.as_tensor(box, dtype=pos.dtype, device=pos.device)
    ri = torch.gather(pos, 1, pairs.i[..., None].expand(-1, -1, 3))
    rj = torch.gather(pos, 1, pairs.j[..., None].expand(-1, -1, 3))
    vi = torch.gather(vel, 1, pairs.i[..., None].expand(-1, -1, 3))
    vj = torch.gather(vel, 1, pairs.j[..., None].expand(-1, -1, 3))
    d = torch.linalg.norm(min_image(rj - ri, box), dim=-1)
    w = bin_weights(d, r_max, bins)
    dots = (vi * vj).sum(-1)
    v2 = (vel ** 2).sum(-1).mean(dim=1, keepdim=True)
    return torch.einsum("rp,rpb->rb", dots, w) / (w.sum(dim=1) + 1e-3) / v2


def loss_s_cv(pos: torch.Tensor, vel: torch.Tensor, L: int, box, pairs: PairSample, cv_target: torch.Tensor,
              s_target: float = 0.7) -> torch.Tensor:
    """(S2 - s_target)^2 + |C_v - C_target|^2, averaged over replicas."""
    t = bead_tangents(pos, L, box)
    S = nematic_s2(t)
    cv = velocity_correlation(pos, vel, pairs, box)
    return ((S - s_target) ** 2).mean() + ((cv - cv_target) ** 2).sum(-1).mean()


def as_rn3(a: torch.Tensor, n_replicas: int) -> torch.Tensor:
    """float4 (N, 4) -> (R, nb, 3)."""
    return a[:, :3].reshape(n_replicas, -1, 3)
