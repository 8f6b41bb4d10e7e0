"""ctypes layout of the reference's parameter structs, as taken by the legacy
C-ABI symbols (nematic-worms_gb300/compat/particles_kernel.cuh, same member
order as simulation/particles_kernel.cuh:26-73)."""
from __future__ import annotations

import ctypes as C

from .abi import NwConfig

_f3 = C.c_float * 3
_u3 = C.c_uint32 * 3


class SimParams(C.Structure):
    _fields_ = [
        ("gravity", _f3),
        ("particleRadius", C.c_float),
        ("particleMass", C.c_float),
        ("gridSize", _u3),
        ("numCells", C.c_uint32),
        ("origin", _f3),
        ("boxSize", _f3),
        ("cellSize", _f3),
        ("boundaryX", C.c_int),
        ("boundaryY", C.c_int),
        ("boundaryZ", C.c_int),
        ("numParticles", C.c_uint32),
        ("numFilaments", C.c_uint32),
        ("filamentSize", C.c_uint32),
        ("bondSpringK", C.c_float),
        ("bondSpringL", C.c_float),
        ("bondBendingK", C.c_float),
        ("activity", C.c_float),
        ("reverseProbability", C.c_float),
        ("kbT", C.c_float),
        ("gamma", C.c_float),
        ("spring", C.c_float),
        ("damping", C.c_float),
        ("shear", C.c_float),
        ("attraction", C.c_float),
        ("boundaryDamping", C.c_float),
    ]

    @classmethod
    def from_config(cls, c: NwConfig) -> "SimParams":
        p = cls()
        p.gravity = _f3(*c.gravity)
        p.particleRadius = c.radius
        p.particleMass = c.mass
        p.gridSize = _u3(*c.grid)
        p.numCells = c.n_cells
        p.origin = _f3(*c.origin)
        p.boxSize = _f3(*c.box)
        p.cellSize = _f3(*c.cell_size)
        p.boundaryX, p.boundaryY, p.boundaryZ = c.boundary[0], c.boundary[1], c.boundary[2]
        p.numParticles = c.n_beads
        p.numFilaments = c.num_filaments
        p.filamentSize = c.filament_size
        p.bondSpringK = c.bond_k
        p.bondSpringL = c.bond_r0
        p.bondBendingK = c.bend_k
        p.activity = c.activity
        p.reverseProbability = c.reverse_probability
        p.kbT = c.kT
        p.gamma = c.gamma
        p.spring = c.spring
        p.damping = c.damping
        p.shear = c.shear
        p.attraction = c.attraction
        p.boundaryDamping = c.boundary_damping
        return p


class SolventParams(C.Structure):
    _fields_ = [
        ("enabled", C.c_bool),
        ("gridSize", _u3),
        ("numCells", C.c_uint32),
        ("randOffset", _f3),
        ("cellSize", _f3),
        ("numParticles", C.c_uint32),
        ("alpha", C.c_float),
        ("kbT", C.c_float),
        ("particleMass", C.c_float),
    ]

    @classmethod
    def from_config(cls, c: NwConfig, shift=(0.0, 0.0, 0.0)) -> "SolventParams":
        s = cls()
        s.enabled = bool(c.srd_enabled)
        s.gridSize = _u3(*c.srd_grid)
        s.numCells = c.n_srd_cells
        s.randOffset = _f3(*shift)
        s.cellSize = _f3(*c.srd_cell_size)
        s.numParticles = c.num_solvent
        s.alpha = c.srd_alpha
        s.kbT = c.srd_kT
        s.particleMass = c.solvent_mass
        return s


def set_parameters(lib, cfg: NwConfig, shift=(0.0, 0.0, 0.0)):
    """setParameters + setSolventParameters from a configuration; returns the structs."""
    sp = SimParams.from_config(cfg)
    sv = SolventParams.from_config(cfg, shift)
    lib.setParameters(C.byref(sp))
    lib.setSolventParameters(C.byref(sv))
    return sp, sv
