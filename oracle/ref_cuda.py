"""ctypes wrapper of the reference CUDA build on the GPU (oracle/ref_cuda).

TEST INFRASTRUCTURE ONLY: the reference's own device code, built unmodified
for sm_103a (oracle/_ref/nwref_kernels.fatbin, made from the reference tree by
oracle/ref_cuda/Makefile), driven by the host harness oracle/ref_cuda/
nwref_host.cu (oracle/_build/libnwref_cuda.so, built on each host).  Used by
tests/ as the checker and by bench.py's reference arms as the speed
denominator; the product never imports it.

``Ref`` exposes the reference's C-ABI functions (``calcHash``, ``sortParticles``
... with the reference's argument order, device pointers as ints) and
``RefSystem`` the reference's ParticleSystem buffers and update sequence.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
sys.path.insert(0, str(REPO / "nematic-worms_gb300"))
from nwgb.legacy import SimParams, SolventParams  # noqa: E402  (the reference's struct layout)

HOST_LIB = HERE / "_build" / "libnwref_cuda.so"
FATBIN = HERE / "_ref" / "nwref_kernels.fatbin"

# buffer ids of nwref_system (nwref_host.cu)
POS, VEL, TANGENT, FORCE, FORCE_OLD, RANDOM, SORTED_POS, SORTED_VEL, SORTED_TANGENT, HASH, INDEX, CELL_START, \
    CELL_END, SOLVENT_COM = range(14)

_P = C.c_void_p
_u = C.c_uint32
_f = C.c_float

_SIGS = {
    "nwref_init": [C.c_char_p],
    "nwref_randomizeUniform": [_P, _u],
    "nwref_randomizeGaussian": [_P, _u, _f, _f],
    "nwref_setParameters": [_P],
    "nwref_setSolventParameters": [_P],
    "nwref_integrateFilaments": [_P, _P, _P, _P, _f, _u],
    "nwref_integrateSolvent": [_P, _P, _f, _u, _u],
    "nwref_calcHash": [_P, _P, _P, C.c_int, C.c_bool],
    "nwref_reorderDataAndFindCellStart": [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _u, _u],
    "nwref_collideFilaments": [_P, _P, _P, _P, _P, _P, _P, _u, _u],
    "nwref_collide_solvent_apply": [_P, _P, _P, _P, _u],
    "nwref_collideSolvent": [_P, _P, _P, _P, _u, _u],
    "nwref_filamentForces": [_P, _P, _P, _f],
    "nwref_sortParticles": [_P, _P, _u],
    "nwref_reverse_apply": [_P, _P, _P, _P, _P, _u],
    "nwref_reverseFilaments": [_P, _P, _P, _P, _P, _u],
    "nwref_langevin_apply": [_P, _P, _P, _u],
    "nwref_langevinThermostat": [_P, _P, _P, _f, _f, _u],
    "nwref_solventCellCentorOfMomentum": [_P, _P, _P, _P, _P, _u],
    "nwref_solventIsokineticThermostat": [_P, _P, _P, _P, _P, _u],
    "nwref_create": [_P, _P, _u],
    "nwref_create_reference": [_u, _u, _u, _u, _u, C.c_int],
    "nwref_reset": [_P],
    "nwref_destroy": [_P],
    "nwref_params": [_P],
    "nwref_solvent": [_P],
    "nwref_buffer": [_P, C.c_int],
    "nwref_buffer_bytes": [_P, C.c_int],
    "nwref_update_count": [_P],
    "nwref_copy": [_P, C.c_int, _P, C.c_size_t, C.c_size_t, C.c_int],
    "nwref_update": [_P, _f, _P],
    "nwref_run": [_P, _u, _f, C.POINTER(_f)],
    "nwref_sync": [],
}
_RESTYPES = {"nwref_create": _P, "nwref_create_reference": _P, "nwref_params": C.POINTER(SimParams), "nwref_solvent": C.POINTER(SolventParams),
             "nwref_buffer": _P, "nwref_buffer_bytes": C.c_size_t, "nwref_update_count": C.c_ulonglong,
             "nwref_destroy": None, "nwref_error": C.c_char_p}

_lib = None


def available() -> str | None:
    """None when the harness and the fatbin are both present, else why not."""
    if not FATBIN.exists():
        return f"{FATBIN.name} missing (built from the reference tree by oracle/ref_cuda/Makefile)"
    if not HOST_LIB.exists():
        return f"{HOST_LIB.name} missing: run the build first"
    return None


class RefCudaError(RuntimeError):
    pass


def lib() -> C.CDLL:
    """Load the harness and initialise it on the current device."""
    global _lib
    if _lib is None:
        why = available()
        if why:
            raise FileNotFoundError(why)
        L = C.CDLL(str(HOST_LIB))
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, C.c_int)
        L.nwref_error.restype = C.c_char_p
        L.nwref_error.argtypes = []
        if L.nwref_init(str(FATBIN).encode()) != 0:
            raise RefCudaError(L.nwref_error().decode())
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != 0:
        raise RefCudaError(lib().nwref_error().decode())


class Ref:
    """The reference's C-ABI functions (simulation/particleSystem_cuda.cu:36-371),
    named as there; every call raises on a CUDA / cuRAND error."""

    def __getattr__(self, name):
        fn = getattr(lib(), "nwref_" + name)

        def call(*args):
            check(fn(*args))

        return call

    @staticmethod
    def setParameters(p: SimParams):
        check(lib().nwref_setParameters(C.byref(p)))

    @staticmethod
    def setSolventParameters(s: SolventParams):
        check(lib().nwref_setSolventParameters(C.byref(s)))


class RefSystem:
    """The reference's ParticleSystem buffers (particleSystem.cpp:172-223) and
    update() / _solventUpdate() sequence (:249-413) on the reference kernels."""

    def __init__(self, params: SimParams | None = None, solvent: SolventParams | None = None, solvent_gap: int = 5,
                 reference=None):
        """From parameter blocks, or with reference=(numFilaments, filamentSize,
        (gx, gy, gz), srd) as the reference's constructor builds them."""
        L = lib()
        if reference is not None:
            M, Lf, g, srd = reference
            self._h = L.nwref_create_reference(M, Lf, g[0], g[1], g[2], 1 if srd else 0)
        else:
            self._h = L.nwref_create(C.byref(params), C.byref(solvent) if solvent is not None else None, solvent_gap)
        if not self._h:
            raise RefCudaError(L.nwref_error().decode())
        self.n_beads = int(self.params.numParticles)
        self.n_solvent = int(self.solvent.numParticles) if self.solvent.enabled else 0

    def reset(self) -> None:
        """ParticleSystem::reset: the reference's lattice state, uploaded."""
        check(lib().nwref_reset(self._h))

    @property
    def params(self) -> SimParams:
        return lib().nwref_params(self._h).contents

    @property
    def solvent(self) -> SolventParams:
        return lib().nwref_solvent(self._h).contents

    def ptr(self, which: int) -> int:
        return lib().nwref_buffer(self._h, which)

    def nbytes(self, which: int) -> int:
        return lib().nwref_buffer_bytes(self._h, which)

    def set(self, which: int, data: np.ndarray, offset_bytes: int = 0) -> None:
        a = np.ascontiguousarray(data)
        check(lib().nwref_copy(self._h, which, a.ctypes.data, offset_bytes, a.nbytes, 1))

    def get(self, which: int, dtype=np.float32, count: int | None = None) -> np.ndarray:
        n = self.nbytes(which) // np.dtype(dtype).itemsize if count is None else count
        out = np.empty(n, dtype)
        check(lib().nwref_copy(self._h, which, out.ctypes.data, 0, out.nbytes, 0))
        return out.reshape(-1, 4) if dtype == np.float32 else out

    def update(self, dt: float, shift=None) -> None:
        sh = None if shift is None else (C.c_float * 2)(*shift[:2])
        check(lib().nwref_update(self._h, dt, sh))

    def run(self, n: int, dt: float) -> float:
        """n updates timed with events on the legacy default stream; ms."""
        ms = C.c_float(0.0)
        check(lib().nwref_run(self._h, n, dt, C.byref(ms)))
        return float(ms.value)

    @property
    def update_count(self) -> int:
        return int(lib().nwref_update_count(self._h))

    def close(self) -> None:
        if self._h:
            lib().nwref_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
