"""ctypes wrapper of the CPU oracle (oracle/_build/libnworacle.so) and of the
CPU emulation of the reference's own kernels (oracle/_ref/*.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  Arrays are numpy float4-style
(n, 4) in float32 or float64 and uint32 index arrays; every function works on
copies and returns new arrays.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
sys.path.insert(0, str(REPO / "nematic-worms_gb300"))
from nwgb.abi import NwConfig  # noqa: E402  (the shared configuration layout)

LIB_PATH = HERE / "_build" / "libnworacle.so"
REF_MODERN = HERE / "_ref" / "libnwref_modern.so"
REF_ARCHIVED = HERE / "_ref" / "libnwref_archived.so"

EMPTY = 0xFFFFFFFF
_lib = None
_ref_m = None
_ref_a = None

_P = C.c_void_p
_u32 = C.c_uint32
_u64 = C.c_uint64
_CP = C.POINTER(NwConfig)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise FileNotFoundError(f"{LIB_PATH} missing: run the build first")
        L = C.CDLL(str(LIB_PATH))
        L.nwo_philox4x32_10.argtypes = [_P, _P, _P]
        L.nwo_u01.restype = C.c_float
        L.nwo_u01.argtypes = [_u32]
        L.nwo_normal4.argtypes = [_u64, _u32, _u64, _u32, _P]
        L.nwo_uniform4.argtypes = [_u64, _u32, _u64, _u32, _P]
        L.nwo_calc_hash.argtypes = [_CP, _P, _u32, _P, _P]
        L.nwo_calc_hash_srd.argtypes = [_CP, _P, _u32, _P, _P, _P]
        L.nwo_sort_by_key.argtypes = [_P, _P, _u32]
        L.nwo_cell_bounds.argtypes = [_P, _u32, _u32, _P, _P]
        L.nwo_num_cells.restype = _u32
        L.nwo_num_cells.argtypes = [_CP]
        L.nwo_num_srd_cells.restype = _u32
        L.nwo_num_srd_cells.argtypes = [_CP]
        L.nwo_set_force_scale.argtypes = [_P]
        L.nwo_num_threads.restype = C.c_int
        L.nwo_set_num_threads.argtypes = [C.c_int]
        for s, R in (("f32", C.c_float), ("f64", C.c_double)):
            getattr(L, f"nwo_integrate_{s}").argtypes = [_CP, _P, _P, _P, _P, _u32, R]
            getattr(L, f"nwo_integrate_solvent_{s}").argtypes = [_CP, _P, _P, _u32, _u32, R]
            getattr(L, f"nwo_reverse_{s}").argtypes = [_CP, _P, _P, _P, _P, _P, _u32]
            getattr(L, f"nwo_langevin_{s}").argtypes = [_CP, _P, _P, _P, _u32]
            getattr(L, f"nwo_filament_{s}").argtypes = [_CP, _P, _P, _P, _u32]
            getattr(L, f"nwo_pair_{s}").argtypes = [_CP, _P, _P, _P, _P, _P, _P, _P, _u32]
            getattr(L, f"nwo_pair_wca_bruteforce_{s}").argtypes = [_CP, _P, _P, _u32]
            getattr(L, f"nwo_srd_{s}").argtypes = [_CP, _P, _P, _u32, _u32, _P, _P, _u64, R, _P, _P, _P, _P]
            getattr(L, f"nwo_step_{s}").argtypes = [_CP, _P, _P, _P, _P, _P, _u64, R, _P, _P, _P, _P]
            getattr(L, f"nwo_srd_shift_{s}").argtypes = [_CP, _u64, _P]
            getattr(L, f"nwo_reorder_solvent_{s}").argtypes = [_P, _P, _u32, _u32, _P]
        _lib = L
    return _lib


def _dt(prec):
    return (np.float32, "f32") if prec == 32 else (np.float64, "f64")


def _f4(a, dtype):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype).reshape(-1, 4)).copy()


def _u(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32).reshape(-1)).copy()


def _ptr(a):
    return None if a is None else a.ctypes.data


# ---- RNG ---------------------------------------------------------------------

def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().nwo_philox4x32_10(c, k, o)
    return list(o)


def normal4(seed, index, step, stream):
    o = (C.c_double * 4)()
    lib().nwo_normal4(seed, index, step, stream, o)
    return np.array(list(o))


def uniform4(seed, index, step, stream):
    o = (C.c_float * 4)()
    lib().nwo_uniform4(seed, index, step, stream, o)
    return np.array(list(o), dtype=np.float32)


# ---- hashing / sorting ---------------------------------------------------------

def calc_hash(cfg: NwConfig, pos):
    p = _f4(pos, np.float32)
    n = p.shape[0]
    h = np.empty(n, np.uint32)
    i = np.empty(n, np.uint32)
    lib().nwo_calc_hash(C.byref(cfg), _ptr(p), n, _ptr(h), _ptr(i))
    return h, i


def calc_hash_srd(cfg: NwConfig, pos, shift):
    p = _f4(pos, np.float32)
    n = p.shape[0]
    h = np.empty(n, np.uint32)
    i = np.empty(n, np.uint32)
    s = np.asarray(shift, dtype=np.float32)
    lib().nwo_calc_hash_srd(C.byref(cfg), _ptr(p), n, _ptr(s), _ptr(h), _ptr(i))
    return h, i


def sort_by_key(keys, values):
    k, v = _u(keys), _u(values)
    lib().nwo_sort_by_key(_ptr(k), _ptr(v), k.shape[0])
    return k, v


def cell_bounds(sorted_hash, num_cells):
    h = _u(sorted_hash)
    cs = np.empty(num_cells, np.uint32)
    ce = np.full(num_cells, EMPTY, np.uint32)
    lib().nwo_cell_bounds(_ptr(h), h.shape[0], num_cells, _ptr(cs), _ptr(ce))
    return cs, ce


def bead_sort(cfg: NwConfig, pos):
    """hash -> stable sort -> cell bounds of bead positions."""
    h, i = calc_hash(cfg, pos)
    sh, si = sort_by_key(h, i)
    cs, ce = cell_bounds(sh, cfg.n_cells)
    return dict(hash=h, sorted_hash=sh, sorted_index=si, cell_start=cs, cell_end=ce)


# ---- physics ---------------------------------------------------------------------

class force_scale:
    """Collects the per-bead force scale (sum of force-term magnitudes before
    cancellation, float64) of the oracle calls made inside the block:
    ``with force_scale(n) as S: pair(...)`` leaves it in S.values."""

    def __init__(self, n: int):
        self.values = np.zeros(max(int(n), 1), np.float64)

    def __enter__(self):
        lib().nwo_set_force_scale(_ptr(self.values))
        return self

    def __exit__(self, *exc):
        lib().nwo_set_force_scale(None)
        return False


def integrate(cfg, pos, vel, force, force_old, dt, prec=32):
    dt_, s = _dt(prec)
    p, v, f, fo = (_f4(a, dt_) for a in (pos, vel, force, force_old))
    getattr(lib(), f"nwo_integrate_{s}")(C.byref(cfg), _ptr(p), _ptr(v), _ptr(f), _ptr(fo), p.shape[0], dt)
    return p, v, f, fo


def integrate_solvent(cfg, pos, vel, start, count, dt, prec=32):
    dt_, s = _dt(prec)
    p, v = _f4(pos, dt_), _f4(vel, dt_)
    getattr(lib(), f"nwo_integrate_solvent_{s}")(C.byref(cfg), _ptr(p), _ptr(v), start, count, dt)
    return p, v


def reverse(cfg, force, force_old, vel, pos, uniform, prec=32):
    dt_, s = _dt(prec)
    f, fo, v, p = (_f4(a, dt_) for a in (force, force_old, vel, pos))
    u = np.ascontiguousarray(np.asarray(uniform, dtype=np.float32))
    getattr(lib(), f"nwo_reverse_{s}")(C.byref(cfg), _ptr(f), _ptr(fo), _ptr(v), _ptr(p), _ptr(u), u.shape[0])
    return f, fo, v, p


def langevin(cfg, force, vel, noise, prec=32):
    dt_, s = _dt(prec)
    f, v, z = _f4(force, dt_), _f4(vel, dt_), _f4(noise, dt_)
    getattr(lib(), f"nwo_langevin_{s}")(C.byref(cfg), _ptr(f), _ptr(v), _ptr(z), f.shape[0])
    return f


def filament(cfg, force, tangent, pos, prec=32):
    dt_, s = _dt(prec)
    f, t, p = _f4(force, dt_), _f4(tangent, dt_), _f4(pos, dt_)
    getattr(lib(), f"nwo_filament_{s}")(C.byref(cfg), _ptr(f), _ptr(t), _ptr(p), cfg.num_filaments)
    return f, t


def pair(cfg, force, pos, vel, tangent, sorted_index, cell_start, cell_end, prec=32):
    dt_, s = _dt(prec)
    f, p, v, t = (_f4(a, dt_) for a in (force, pos, vel, tangent))
    si, cs, ce = _u(sorted_index), _u(cell_start), _u(cell_end)
    getattr(lib(), f"nwo_pair_{s}")(C.byref(cfg), _ptr(f), _ptr(p), _ptr(v), _ptr(t), _ptr(si), _ptr(cs), _ptr(ce),
                                    si.shape[0])
    return f


def pair_wca_bruteforce(cfg, force, pos, prec=64):
    dt_, s = _dt(prec)
    f, p = _f4(force, dt_), _f4(pos, dt_)
    getattr(lib(), f"nwo_pair_wca_bruteforce_{s}")(C.byref(cfg), _ptr(f), _ptr(p), p.shape[0])
    return f


def srd(cfg, pos, vel, n_beads, n_solvent, shift, rot_uniform=None, step=0, dt_srd=0.0, prec=32):
    dt_, s = _dt(prec)
    p, v = _f4(pos, dt_), _f4(vel, dt_)
    C_ = int(lib().nwo_num_srd_cells(C.byref(cfg)))
    n = n_beads + n_solvent
    si = np.empty(n, np.uint32)
    cs = np.empty(C_, np.uint32)
    ce = np.empty(C_, np.uint32)
    cm = np.empty((C_, 4), dt_)
    sh = np.asarray(shift, dtype=np.float32)
    ru = None if rot_uniform is None else np.ascontiguousarray(np.asarray(rot_uniform, dtype=np.float32))
    getattr(lib(), f"nwo_srd_{s}")(C.byref(cfg), _ptr(p), _ptr(v), n_beads, n_solvent, _ptr(sh), _ptr(ru), step,
                                   dt_srd, _ptr(si), _ptr(cs), _ptr(ce), _ptr(cm))
    return dict(pos=p, vel=v, sorted_index=si, cell_start=cs, cell_end=ce, cell_mean=cm)


def reorder_solvent(pos, vel, n_beads, n_solvent, sorted_index, prec=32):
    """Solvent relabelled in the collision's stable cell order (the order the
    engine stores it in after a collision); beads unchanged."""
    dt_, s = _dt(prec)
    p, v = _f4(pos, dt_), _f4(vel, dt_)
    si = np.ascontiguousarray(np.asarray(sorted_index, dtype=np.uint32))
    getattr(lib(), f"nwo_reorder_solvent_{s}")(_ptr(p), _ptr(v), n_beads, n_solvent, _ptr(si))
    return p, v


def srd_shift(cfg, step, prec=32):
    o = (C.c_float * 3)()
    getattr(lib(), f"nwo_srd_shift_{_dt(prec)[1]}")(C.byref(cfg), step, o)
    return np.array(list(o), dtype=np.float32)


def step(cfg, state, step_index, dt, prec=32, force_scale=False):
    """One full step; state = dict(pos, vel, force, force_old, tangent).
    With force_scale, the result also holds ``force_scale``: per bead the sum
    of the magnitudes of every force term of the step (float64), the scale
    that bounds the rounding error of the bead's net force."""
    dt_, s = _dt(prec)
    p, v, f, fo, t = (_f4(state[k], dt_) for k in ("pos", "vel", "force", "force_old", "tangent"))
    nb = cfg.n_beads
    nc = int(lib().nwo_num_cells(C.byref(cfg)))
    h = np.empty(nb, np.uint32)
    si = np.empty(nb, np.uint32)
    cs = np.empty(nc, np.uint32)
    ce = np.empty(nc, np.uint32)
    fs = np.zeros(max(nb, 1), np.float64) if force_scale else None
    lib().nwo_set_force_scale(_ptr(fs))
    try:
        getattr(lib(), f"nwo_step_{s}")(C.byref(cfg), _ptr(p), _ptr(v), _ptr(f), _ptr(fo), _ptr(t), step_index, dt,
                                        _ptr(h), _ptr(si), _ptr(cs), _ptr(ce))
    finally:
        lib().nwo_set_force_scale(None)
    out = dict(pos=p, vel=v, force=f, force_old=fo, tangent=t, hash=h, sorted_index=si, cell_start=cs, cell_end=ce)
    if force_scale:
        out["force_scale"] = fs[:nb]
    return out


def set_threads(n: int) -> None:
    lib().nwo_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().nwo_num_threads())


# ---- the reference's own kernels, emulated on the CPU ---------------------------------

def have_reference() -> bool:
    return REF_MODERN.exists() and REF_ARCHIVED.exists()


def ref_modern() -> C.CDLL:
    global _ref_m
    if _ref_m is None:
        L = C.CDLL(str(REF_MODERN))
        L.ref_calc_hash.argtypes = [_CP, _P, _P, _P, _P, _u32, C.c_int]
        L.ref_reorder.argtypes = [_CP, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _u32, _u32]
        L.ref_collide_filaments.argtypes = [_CP, _P, _P, _P, _P, _P, _P, _P, _u32]
        L.ref_filament_forces.argtypes = [_CP, _P, _P, _P, _u32]
        L.ref_langevin.argtypes = [_CP, _P, _P, _P, _u32]
        L.ref_integrate.argtypes = [_CP, _P, _P, _P, _P, C.c_float, _u32]
        L.ref_integrate_solvent.argtypes = [_CP, _P, _P, C.c_float, _u32, _u32]
        L.ref_reverse.argtypes = [_CP, _P, _P, _P, _P, _P, _u32]
        L.ref_srd_thermostat.argtypes = [_CP, _P, _P, _P, _P, _P, _u32]
        L.ref_srd_com.argtypes = [_CP, _P, _P, _P, _P, _P, _u32]
        L.ref_collide_solvent.argtypes = [_CP, _P, _P, _P, _P, _P, _u32]
        L.ref_sizeof_simparams.restype = C.c_size_t
        _ref_m = L
    return _ref_m


def ref_archived() -> C.CDLL:
    global _ref_a
    if _ref_a is None:
        L = C.CDLL(str(REF_ARCHIVED))
        L.ref_archived_forces.restype = C.c_int
        L.ref_archived_forces.argtypes = [_CP, _P, _P, _P, C.c_float, _P]
        L.ref_archived_lj_constants.argtypes = [C.c_float, C.c_float, _P]
        _ref_a = L
    return _ref_a
