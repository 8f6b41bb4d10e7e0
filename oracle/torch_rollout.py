"""FP64 restatement of the adjoint rollout in torch on the CPU, with autograd.
TEST INFRASTRUCTURE ONLY: the reference gradient and the finite-difference
forward the CUDA adjoint (include/nwgb_adjoint.h) is checked against.

Same step and conventions as the CUDA rollout: velocity Verlet in the
engine's ordering (simulation/particles_kernel_impl.cuh:93-97), Langevin
(:859-874) with the Philox noise of the oracle (nw_oracle.h nwo_normal4),
bending (:751-818), archived WCA laws (NWWormsKernel_LennardJones.h:38-50,
NWWormsKernel_InternalForce.h:37-59, NWWormsKernel_DriveForce.h:21-34),
neighbour lists frozen per segment (all non-excluded pairs within
lj_rcut + skin at the segment's start).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

import oracle as orc


def noise_table(cfg, n_replicas: int, horizon: int) -> np.ndarray:
    """sigma * xi for every update m (counter m - 1), replica and bead: (H, N, 3)."""
    nb = cfg.n_beads
    s2 = 2.0 * cfg.gamma * cfg.kT
    if cfg.noise_dt_scaling:
        s2 /= cfg.dt
    sigma = math.sqrt(s2)
    out = np.zeros((horizon, n_replicas * nb, 3))
    buf = (C.c_double * 4)()
    lib = orc.lib()
    for m in range(horizon):
        for r in range(n_replicas):
            for i in range(nb):
                lib.nwo_normal4(C.c_uint64(cfg.seed + r), i, m, 1, buf)
                out[m, r * nb + i, 0] = buf[0]
                out[m, r * nb + i, 1] = buf[1]
                if cfg.dim >= 3:
                    out[m, r * nb + i, 2] = buf[2]
    return sigma * out


def _min_image(d, box):
    half = box / 2
    return torch.where(d > half, d - box, torch.where(d < -half, d + box, d))


def frozen_pairs(cfg, r: np.ndarray, n_replicas: int):
    """(I, J) of all ordered pairs on the lists built from positions r (N, 3)."""
    nb, L = cfg.n_beads, cfg.filament_size
    skin = cfg.neighbor_skin if cfg.neighbor_skin > 0 else 0.3 * cfg.lj_sigma
    rl2 = (cfg.lj_rcut + skin) ** 2
    box = np.array([cfg.box[0], cfg.box[1], cfg.box[2]])
    I, J = [], []
    for rep in range(n_replicas):
        p = r[rep * nb:(rep + 1) * nb]
        for a in range(nb):
            d = p - p[a]
            d = np.where(d > box / 2, d - box, np.where(d < -box / 2, d + box, d))
            q = (d * d).sum(1)
            ok = q <= rl2
            ok[a] = False
            idx = np.nonzero(ok)[0]
            same = (idx // L) == (a // L)
            idx = idx[~(same & (np.abs(idx - a) <= cfg.lj_exclude))]
            I.append(np.full(idx.size, rep * nb + a))
            J.append(rep * nb + idx)
    return torch.from_numpy(np.concatenate(I)), torch.from_numpy(np.concatenate(J))


def forces(cfg, theta, r, v, xi, pairs):
    eps, kbend, kbond, fact = theta[0], theta[1], theta[2], theta[3]
    N = r.shape[0]
    L = cfg.filament_size
    box = torch.tensor([cfg.box[0], cfg.box[1], cfg.box[2]], dtype=r.dtype)
    F = -cfg.gamma * v + xi
    R4 = r.reshape(-1, L, 3)
    # bending triples (p, p+1, p+2)
    if L >= 3:
        a = _min_image(R4[:, 1:-1] - R4[:, :-2], box)
        b = _min_image(R4[:, 2:] - R4[:, 1:-1], box)
        qa, qb = (a * a).sum(-1, keepdim=True), (b * b).sum(-1, keepdim=True)
        dd = (a * b).sum(-1, keepdim=True)
        A = 1.0 / torch.sqrt(qa * qb)
        fi = -A * (b - a * (dd / qa))
        fk = -A * (b * (dd / qb) - a)
        fj = -fi - fk
        pad = torch.nn.functional.pad
        Fb = pad(fi, (0, 0, 0, 2)) + pad(fj, (0, 0, 1, 1)) + pad(fk, (0, 0, 2, 0))
        F = F + kbend * Fb.reshape(N, 3)
    # bonds (on both beads) and drive (on the first bead of each bond)
    d = _min_image(R4[:, 1:] - R4[:, :-1], box)
    dl = torch.sqrt((d * d).sum(-1, keepdim=True))
    fb = kbond * (1.0 - cfg.bond_r0 / dl) * d
    drive = fact * d / dl
    Fbd = torch.nn.functional.pad(fb + drive, (0, 0, 0, 1)) - torch.nn.functional.pad(fb, (0, 0, 1, 0))
    F = F + Fbd.reshape(N, 3)
    # LJ over the frozen list
    I, J = pairs
    dr = _min_image(r[J] - r[I], box)
    q = (dr * dr).sum(-1, keepdim=True)
    s6 = cfg.lj_sigma ** 6
    iq = 1.0 / q
    fm = 24.0 * s6 * (2.0 * s6 * iq ** 7 - iq ** 4)
    fm = torch.where(q <= cfg.lj_rcut ** 2, fm, torch.zeros_like(fm))
    F = F.index_add(0, I, -eps * fm * dr)
    return F


def rollout(cfg, theta: torch.Tensor, pos0: np.ndarray, vel0: np.ndarray, n_replicas: int, horizon: int,
            segment: int, xi: np.ndarray):
    """Final (r, v) (N, 3) float64 tensors, differentiable in theta."""
    r = torch.tensor(pos0[:, :3], dtype=torch.float64)
    v = torch.tensor(vel0[:, :3], dtype=torch.float64)
    F = torch.zeros_like(r)
    Fo = torch.zeros_like(r)
    dt = cfg.dt
    org = torch.tensor([cfg.origin[0], cfg.origin[1], cfg.origin[2]], dtype=torch.float64)
    box = torch.tensor([cfg.box[0], cfg.box[1], cfg.box[2]], dtype=torch.float64)
    xi_t = torch.from_numpy(xi)
    for s0 in range(0, horizon, segment):
        pairs = frozen_pairs(cfg, r.detach().numpy(), n_replicas)
        for m in range(s0 + 1, min(horizon, s0 + segment) + 1):
            v = v + 0.5 * dt * (F + Fo)
            r = r + dt * v + 0.5 * dt * dt * F
            r = torch.where(r < org, r + box, torch.where(r > org + box, r - box, r))
            Fo = F
            F = forces(cfg, theta, r, v, xi_t[m - 1], pairs)
    return r, v
