"""ctypes view of the C ABI in include/nwgb.h and include/nw_legacy.h.

The shared library is built in-tree (nematic-worms_gb300/lib/libnwgb.so) by
``nwgb.build_library``.  Loading fails loudly when it is missing: there is no
fallback implementation of the step.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_ROOT = Path(__file__).resolve().parent.parent          # nematic-worms_gb300/
REPO_ROOT = PKG_ROOT.parent
LIB_DIR = PKG_ROOT / "lib"
LIB_PATH = LIB_DIR / "libnwgb.so"

NW_ABI_VERSION = 2

# status codes
NW_OK = 0
NW_ERR_CUDA = 1
NW_ERR_INVALID = 2
NW_ERR_CELL_OVERFLOW = 3
NW_ERR_NONFINITE = 4
NW_ERR_TIMEOUT = 5
NW_ERR_NOMEM = 6
NW_ERR_UNSUPPORTED = 7
NW_ERR_NO_DEVICE = 8
NW_ERR_IO = 9

NW_EFLAG_NONFINITE = 1 << 0
NW_EFLAG_CELL_OVERFLOW = 1 << 1
NW_EFLAG_TIMEOUT = 1 << 2
NW_EFLAG_BAD_INDEX = 1 << 3
NW_EFLAG_NEIGHBOR_OVERFLOW = 1 << 4

NW_MODEL_WCA_WORMS = 0
NW_MODEL_REF_DEM = 1
NW_PERIODIC, NW_WALL, NW_WALL_NO_SLIP = 0, 1, 2
NW_HASH_MODULO, NW_HASH_MASK = 0, 1
NW_SRD_THERMO_NONE, NW_SRD_THERMO_REF_LAB, NW_SRD_THERMO_CELL_REL = 0, 1, 2
NW_STRATEGY_AUTO, NW_STRATEGY_SORTED, NW_STRATEGY_CELL_LISTS, NW_STRATEGY_VERLET = 0, 1, 2, 3

NW_POSITION = 0
NW_VELOCITY = 1
NW_TANGENT = 2
NW_FORCE = 3
NW_FORCE_OLD = 4
NW_HASH = 5
NW_SORTED_INDEX = 6
NW_CELL_START = 7
NW_CELL_END = 8
NW_SRD_SORTED_INDEX = 9
NW_SRD_CELL_START = 10
NW_SRD_CELL_END = 11
NW_SRD_CELL_MEAN = 12

EMPTY = 0xFFFFFFFF

_u32 = C.c_uint32
_i32 = C.c_int32
_f32 = C.c_float


class NwConfig(C.Structure):
    """Mirror of ``struct NwConfig`` (include/nwgb.h)."""

    _fields_ = [
        ("abi_version", _u32),
        ("model", _i32),
        ("dim", _i32),
        ("num_filaments", _u32),
        ("filament_size", _u32),
        ("grid", _u32 * 3),
        ("cell_size", _f32 * 3),
        ("origin", _f32 * 3),
        ("box", _f32 * 3),
        ("boundary", _i32 * 3),
        ("hash_mode", _i32),
        ("radius", _f32),
        ("mass", _f32),
        ("bond_k", _f32),
        ("bond_r0", _f32),
        ("bend_k", _f32),
        ("lj_epsilon", _f32),
        ("lj_sigma", _f32),
        ("lj_rcut", _f32),
        ("lj_exclude", _i32),
        ("spring", _f32),
        ("damping", _f32),
        ("shear", _f32),
        ("attraction", _f32),
        ("boundary_damping", _f32),
        ("activity", _f32),
        ("reverse_probability", _f32),
        ("gamma", _f32),
        ("kT", _f32),
        ("noise_dt_scaling", _i32),
        ("langevin_with_srd", _i32),
        ("gravity", _f32 * 3),
        ("srd_enabled", _i32),
        ("num_solvent", _u32),
        ("srd_grid", _u32 * 3),
        ("srd_cell_size", _f32 * 3),
        ("srd_alpha", _f32),
        ("srd_gap", _u32),
        ("srd_kT", _f32),
        ("solvent_mass", _f32),
        ("srd_shift_lo", _f32),
        ("srd_rotate_beads", _i32),
        ("srd_thermostat", _i32),
        ("seed", C.c_uint64),
        ("dt", _f32),
        ("strategy", _i32),
        ("cell_capacity", _u32),
        ("neighbor_skin", _f32),
        ("neighbor_capacity", _u32),
        ("reserved", _u32 * 3),
    ]

    def copy(self) -> "NwConfig":
        c = NwConfig()
        C.memmove(C.byref(c), C.byref(self), C.sizeof(NwConfig))
        return c

    @property
    def n_beads(self) -> int:
        return int(self.num_filaments) * int(self.filament_size)

    @property
    def n_solvent(self) -> int:
        return int(self.num_solvent) if self.srd_enabled else 0

    @property
    def n_cells(self) -> int:
        return int(self.grid[0]) * int(self.grid[1]) * int(self.grid[2])

    @property
    def n_srd_cells(self) -> int:
        return int(self.srd_grid[0]) * int(self.srd_grid[1]) * int(self.srd_grid[2])


class NwKernelTime(C.Structure):
    """Mirror of ``struct NwKernelTime`` (include/nwgb.h)."""

    _fields_ = [("name", C.c_char * 32), ("total_ms", C.c_double), ("launches", C.c_uint64)]


class NwError(RuntimeError):
    """A libnwgb call returned a non-OK nw_status."""

    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = STATUS_NAMES.get(status, f"status {status}")
        super().__init__(f"{what}: {msg}" if what else msg)


STATUS_NAMES = {
    NW_OK: "ok",
    NW_ERR_CUDA: "CUDA runtime error",
    NW_ERR_INVALID: "invalid argument or configuration",
    NW_ERR_CELL_OVERFLOW: "cell occupancy above kernel capacity",
    NW_ERR_NONFINITE: "non-finite position or force",
    NW_ERR_TIMEOUT: "bounded device wait timed out",
    NW_ERR_NOMEM: "out of memory",
    NW_ERR_UNSUPPORTED: "unsupported configuration",
    NW_ERR_NO_DEVICE: "no CUDA device",
    NW_ERR_IO: "file could not be opened or written",
}

NW_DEFECT_MIN_IMAGE = 1


class NwDefect(C.Structure):
    """include/nwgb.h NwDefect: one +1/2 or -1/2 defect."""

    _fields_ = [("x", C.c_double), ("y", C.c_double), ("charge", C.c_float), ("cells", _u32)]


class NwObservables(C.Structure):
    """include/nwgb.h NwObservables."""

    _fields_ = [("s_q3", C.c_double), ("s_2d", C.c_double), ("polar", C.c_double),
                ("bead_temperature", C.c_double), ("solvent_temperature", C.c_double), ("msd", C.c_double),
                ("n_beads", _u32), ("n_tangents", _u32), ("n_solvent", _u32), ("reserved", _u32)]


NW_OBS_MIN_IMAGE = 1
NW_OBS_MSD = 2

# numpy view of an NwDefect array (same 24-byte layout)
DEFECT_DTYPE = np.dtype([("x", "<f8"), ("y", "<f8"), ("charge", "<f4"), ("cells", "<u4")])


# Every symbol the library must export: (name, restype, argtypes)
_P = C.c_void_p
_sysp = C.c_void_p
HANDLE_API = [
    ("nw_config_default", C.c_int, [C.POINTER(NwConfig), C.c_int, _u32, _u32, _u32, _u32, _u32, C.c_int]),
    ("nw_config_finalize", C.c_int, [C.POINTER(NwConfig)]),
    ("nw_config_validate", C.c_int, [C.POINTER(NwConfig)]),
    ("nw_create", C.c_int, [C.POINTER(NwConfig), C.POINTER(_sysp)]),
    ("nw_destroy", C.c_int, [_sysp]),
    ("nw_set_config", C.c_int, [_sysp, C.POINTER(NwConfig)]),
    ("nw_get_config", C.c_int, [_sysp, C.POINTER(NwConfig)]),
    ("nw_get_counts", C.c_int, [_sysp, C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32)]),
    ("nw_set_array", C.c_int, [_sysp, C.c_int, _P, _u32, _u32]),
    ("nw_get_array", C.c_int, [_sysp, C.c_int, _P, _u32, _u32]),
    ("nw_set_array_async", C.c_int, [_sysp, C.c_int, _P, _u32, _u32]),
    ("nw_get_array_async", C.c_int, [_sysp, C.c_int, _P, _u32, _u32]),
    ("nw_device_array", C.c_int, [_sysp, C.c_int, C.POINTER(_P)]),
    ("nw_zero_forces", C.c_int, [_sysp]),
    ("nw_step", C.c_int, [_sysp, C.c_int, _f32]),
    ("nw_step_prepare", C.c_int, [_sysp, C.c_int, _f32, C.c_uint64]),
    ("nw_reference_reset", C.c_int, [C.POINTER(NwConfig), _P, _P, _P]),
    ("nw_sync", C.c_int, [_sysp]),
    ("nw_error_word", C.c_int, [_sysp, C.POINTER(_u32)]),
    ("nw_get_step", C.c_int, [_sysp, C.POINTER(C.c_uint64)]),
    ("nw_set_step", C.c_int, [_sysp, C.c_uint64]),
    ("nw_set_stream", C.c_int, [_sysp, _P]),
    ("nw_set_graphs", C.c_int, [_sysp, C.c_int]),
    ("nw_srd_collide", C.c_int, [_sysp, _f32, C.POINTER(_f32)]),
    ("nw_checkpoint_size", C.c_int, [_sysp, C.POINTER(C.c_size_t)]),
    ("nw_checkpoint_save", C.c_int, [_sysp, _P, C.c_size_t]),
    ("nw_checkpoint_load", C.c_int, [_sysp, _P, C.c_size_t]),
    ("nw_status_string", C.c_char_p, [C.c_int]),
    ("nw_abi_version", _u32, []),
    ("nw_config_size", C.c_size_t, []),
    ("nw_last_launch_count", C.c_int, [_sysp, C.POINTER(C.c_uint64)]),
    ("nw_profile_steps", C.c_int, [_sysp, C.c_int, _f32, C.POINTER(NwKernelTime), C.c_int, C.POINTER(C.c_int)]),
    ("nw_math_probe", C.c_int, [C.c_void_p, C.c_void_p, _u32, C.c_void_p]),
    ("nw_writer_open", C.c_int, [_sysp, C.c_char_p, C.c_int, C.POINTER(_P)]),
    ("nw_writer_frame", C.c_int, [_P, C.c_int, _f32]),
    ("nw_writer_flush", C.c_int, [_P]),
    ("nw_writer_close", C.c_int, [_P]),
    ("nw_find_defects", C.c_int, [_sysp, _f32, _u32, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    ("nw_sample_defects", C.c_int, [_sysp, C.c_void_p, C.c_int, _f32, _u32, C.c_void_p]),
    ("nw_observe", C.c_int, [_sysp, _u32, C.POINTER(NwObservables)]),
    ("nw_observe_reset", C.c_int, [_sysp]),
    ("nw_velocity_correlation", C.c_int, [_sysp, _P, _P, _u32, _f32, _u32, _P, _P]),
    ("nw_srd_temperature_histogram", C.c_int, [_sysp, _P, _f32, _u32, _P]),
]

_fp = C.c_void_p  # device pointers are passed as integers
LEGACY_API = [
    ("cudaInit", None, [C.c_int, C.POINTER(C.c_char_p)]),
    ("randomizeUniform", None, [_fp, _u32]),
    ("randomizeGaussian", None, [_fp, _u32, _f32, _f32]),
    ("allocateArray", None, [C.POINTER(_P), C.c_int]),
    ("freeArray", None, [_fp]),
    ("threadSync", None, []),
    ("copyArrayFromDevice", None, [_P, _fp, _P, C.c_int]),
    ("copyArrayToDevice", None, [_fp, _P, C.c_int, C.c_int]),
    ("setParameters", None, [_P]),
    ("setSolventParameters", None, [_P]),
    ("integrateFilaments", None, [_fp, _fp, _fp, _fp, _f32, _u32]),
    ("integrateSolvent", None, [_fp, _fp, _f32, _u32, _u32]),
    ("calcHash", None, [_fp, _fp, _fp, C.c_int, C.c_bool]),
    ("reorderDataAndFindCellStart", None, [_fp, _fp, _fp, _fp, _fp, _fp, _fp, _fp, _fp, _fp, _u32, _u32]),
    ("collideFilaments", None, [_fp, _fp, _fp, _fp, _fp, _fp, _fp, _u32, _u32]),
    ("collideSolvent", None, [_fp, _fp, _fp, _fp, _u32, _u32]),
    ("filamentForces", None, [_fp, _fp, _fp, _f32]),
    ("sortParticles", None, [_fp, _fp, _u32]),
    ("nw_sort_particles_noalloc", C.c_int, [_fp, _fp, _u32]),
    ("reverseFilaments", None, [_fp, _fp, _fp, _fp, _fp, _u32]),
    ("langevinThermostat", None, [_fp, _fp, _fp, _f32, _f32, _u32]),
    ("solventCellCentorOfMomentum", None, [_fp, _fp, _fp, _fp, _fp, _u32]),
    ("solventIsokineticThermostat", None, [_fp, _fp, _fp, _fp, _fp, _u32]),
    ("nw_legacy_last_status", C.c_int, []),
    ("nw_legacy_seed", None, [C.c_uint64]),
    ("nw_legacy_langevin_apply", None, [_fp, _fp, _fp, _u32]),
    ("nw_legacy_reverse_apply", None, [_fp, _fp, _fp, _fp, _fp, _u32]),
    ("nw_legacy_collide_solvent_apply", None, [_fp, _fp, _fp, _fp, _u32]),
]

_lib = None


class NwBatchTuning(C.Structure):
    """include/nwgb_batch.h NwBatchTuning."""

    _fields_ = [("threads_per_block", _u32), ("strategy", C.c_int32), ("neighbor_skin", _f32),
                ("ms_per_step", _f32), ("cell_capacity", _u32)]


_bp = C.c_void_p
BATCH_API = [
    ("nw_batch_create", C.c_int, [C.POINTER(NwConfig), C.c_int, C.POINTER(_bp)]),
    ("nw_batch_destroy", C.c_int, [_bp]),
    ("nw_batch_counts", C.c_int, [_bp, C.POINTER(C.c_int), C.POINTER(C.c_uint64)]),
    ("nw_batch_replica", C.c_int, [_bp, C.c_int, C.POINTER(_u32), C.POINTER(C.c_uint64)]),
    ("nw_batch_set_array", C.c_int, [_bp, C.c_int, C.c_int, _P, _u32, _u32]),
    ("nw_batch_get_array", C.c_int, [_bp, C.c_int, C.c_int, _P, _u32, _u32]),
    ("nw_batch_device_array", C.c_int, [_bp, C.c_int, C.POINTER(_P)]),
    ("nw_batch_step", C.c_int, [_bp, C.c_int]),
    ("nw_batch_sync", C.c_int, [_bp]),
    ("nw_batch_set_stream", C.c_int, [_bp, _P]),
    ("nw_batch_set_graphs", C.c_int, [_bp, C.c_int]),
    ("nw_batch_get_step", C.c_uint64, [_bp]),
    ("nw_batch_last_launch_count", C.c_int, [_bp, C.POINTER(C.c_uint64)]),
    ("nw_batch_get_tuning", C.c_int, [_bp, C.POINTER(NwBatchTuning)]),
    ("nw_batch_set_tuning", C.c_int, [_bp, C.POINTER(NwBatchTuning)]),
    ("nw_batch_autotune", C.c_int, [_bp, C.c_int, C.POINTER(NwBatchTuning)]),
    ("nw_batch_tuning_class", C.c_int, [_bp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
]


_ap = C.c_void_p
ADJOINT_API = [
    ("nw_adj_create", C.c_int, [C.POINTER(NwConfig), C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_ap)]),
    ("nw_adj_destroy", C.c_int, [_ap]),
    ("nw_adj_set_stream", C.c_int, [_ap, _P]),
    ("nw_adj_set_state", C.c_int, [_ap, _P, _P]),
    ("nw_adj_forward", C.c_int, [_ap, C.POINTER(C.c_double), _P, _P]),
    ("nw_adj_backward", C.c_int, [_ap, _P, _P, C.POINTER(C.c_double)]),
    ("nw_adj_final_state_f64", C.c_int, [_ap, _P, _P]),
    ("nw_adj_timings", C.c_int, [_ap, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
]


def load_library(path: os.PathLike | str | None = None) -> C.CDLL:
    """Load libnwgb.so (once) and declare every exported function.

    Raises FileNotFoundError when the library has not been built: the engine
    has no CPU fallback.
    """
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} is missing: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()')"
        )
    lib = C.CDLL(str(p))
    for name, res, args in HANDLE_API + LEGACY_API + BATCH_API + ADJOINT_API:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.nw_abi_version() != NW_ABI_VERSION:
        raise RuntimeError("libnwgb ABI version mismatch")
    if lib.nw_config_size() != C.sizeof(NwConfig):
        raise RuntimeError(f"NwConfig layout mismatch: C {lib.nw_config_size()} vs ctypes {C.sizeof(NwConfig)}")
    if path is None:
        _lib = lib
    return lib


def check(status: int, what: str = "") -> None:
    if status != NW_OK:
        raise NwError(status, what)


def default_config(model: int, num_filaments: int, filament_size: int, grid=(128, 128, 1), srd: bool = False,
                   lib: C.CDLL | None = None) -> NwConfig:
    """nw_config_default: reference (REF_DEM) or WCA worm defaults for a grid."""
    lib = lib or load_library()
    c = NwConfig()
    check(lib.nw_config_default(C.byref(c), model, num_filaments, filament_size, grid[0], grid[1], grid[2],
                                1 if srd else 0), "nw_config_default")
    return c
