"""ParticleSystem::reset (simulation/particleSystem.cpp:583-678) as the
library restates it in C (nw_reference_reset), against a loop-by-loop Python
restatement of the same lines with the same rand() stream.  No GPU."""
from __future__ import annotations

import ctypes as C
import ctypes.util
import math

import numpy as np
import pytest

from nwgb import abi
from nwgb.init import reference_reset


def python_reset(cfg):
    """The reference's reset(), bead by bead, in float32 as the reference
    computes it: rand() after srand(1), frand() = rand() / RAND_MAX."""
    libc = C.CDLL(ctypes.util.find_library("c"))
    libc.rand.restype = C.c_int
    libc.srand(1)
    RAND_MAX = 2147483647.0

    def frand():
        return np.float32(libc.rand()) / np.float32(RAND_MAX)

    nb, ns = cfg.n_beads, cfg.n_solvent
    L, M = int(cfg.filament_size), int(cfg.num_filaments)
    R = np.float32(cfg.radius)
    bl = np.float32(cfg.bond_r0)
    box = np.array(cfg.box, dtype=np.float32)
    org = np.array(cfg.origin, dtype=np.float32)
    flen = np.float32(np.float32(L) * bl + np.float32(2.0) * R)
    xdim = int(math.floor(box[0] / flen))
    ydim = int(math.floor(box[1] / (2 * R)))
    plane = xdim * ydim
    pos = np.zeros((nb + ns, 4), dtype=np.float32)
    vel = np.zeros((nb + ns, 4), dtype=np.float32)
    tan = np.zeros((nb, 4), dtype=np.float32)
    for i in range(nb):
        w = i // L
        x_head = np.float32(w % xdim) * flen + R
        x = x_head + np.float32(i % L) * bl
        y = np.float32(2.0) * R * np.float32((w // xdim) % ydim + 1)
        z = np.float32(2.0) * R * np.float32(w // plane + 1)
        pos[i] = (x + org[0], y + org[1], z + org[2], R)
        vel[i, 0] = np.float32(0.1) * (frand() * np.float32(2.0) - np.float32(1.0))
        vel[i, 1] = np.float32(0.1) * (frand() * np.float32(2.0) - np.float32(1.0))
        vel[i, 2] = np.float32(0.1) * (frand() * np.float32(2.0) - np.float32(1.0))
        vel[i, 3] = cfg.mass
        tan[i] = (1.0, 0.0, 0.0, 0.0)
    for w in range(M):
        if frand() < np.float32(0.5):
            continue
        for p in range(L // 2):
            i, j = w * L + p, (w + 1) * L - 1 - p
            pos[[i, j]] = pos[[j, i]]
            tan[i] = -tan[i]
            tan[j] = -tan[j]
    for s in range(ns):
        i = nb + s
        pos[i, 0] = box[0] * frand() + org[0]
        pos[i, 1] = box[1] * frand() + org[1]
        pos[i, 2] = box[2] * frand() + org[2]
        pos[i, 3] = 0.0
        v0 = np.float32(5.0)
        vel[i, 0] = v0 * (frand() * np.float32(2.0) - np.float32(1.0))
        vel[i, 1] = v0 * (frand() * np.float32(2.0) - np.float32(1.0))
        vel[i, 2] = v0 * (frand() * np.float32(2.0) - np.float32(1.0))
        vel[i, 3] = cfg.solvent_mass
    return pos, vel, tan


@pytest.mark.parametrize("model,M,L,grid,srd", [(abi.NW_MODEL_REF_DEM, 150, 10, (64, 64, 1), True),
                                                 (abi.NW_MODEL_REF_DEM, 37, 7, (32, 16, 4), False)])
def test_reference_reset_matches_restatement(lib, model, M, L, grid, srd):
    cfg = abi.default_config(model, M, L, grid, srd, lib)
    cfg.bond_r0 = 0.8
    a = reference_reset(cfg, lib)
    b = python_reset(cfg)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    # the same draw twice: rand() is reseeded
    c = reference_reset(cfg, lib)
    assert np.array_equal(a[0], c[0])
