"""Host-side mirror of the engine's C ABI.

``System`` wraps the handle API of include/nwgb.h (one simulated system on
one GPU).  ``ParticleSystem`` mirrors the reference's host class
(simulation/particleSystem.h:24-211): same method names, argument meaning and
defaults, so scripts written against the reference read the same here.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import NwConfig, check

_FLOAT4 = {abi.NW_POSITION, abi.NW_VELOCITY, abi.NW_TANGENT, abi.NW_FORCE, abi.NW_FORCE_OLD, abi.NW_SRD_CELL_MEAN}


class System:
    """One system on the current CUDA device (nw_create / nw_destroy)."""

    def __init__(self, cfg: NwConfig, lib: C.CDLL | None = None):
        self.lib = lib or abi.load_library()
        self._h = C.c_void_p()
        check(self.lib.nw_create(C.byref(cfg), C.byref(self._h)), "nw_create")
        nb, ns, nc, nsc = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(self.lib.nw_get_counts(self._h, C.byref(nb), C.byref(ns), C.byref(nc), C.byref(nsc)))
        self.n_beads, self.n_solvent, self.n_cells, self.n_srd_cells = nb.value, ns.value, nc.value, nsc.value

    # -- lifetime -----------------------------------------------------------------
    def close(self) -> None:
        if self._h:
            check(self.lib.nw_destroy(self._h), "nw_destroy")
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def writer(self, path, append: bool = False):
        """Trajectory writer of this system (nwgb.trajectory.Writer)."""
        from .trajectory import Writer

        return Writer(self, path, append)

    def __exit__(self, *exc):
        self.close()

    # -- configuration ----------------------------------------------------------------
    @property
    def config(self) -> NwConfig:
        c = NwConfig()
        check(self.lib.nw_get_config(self._h, C.byref(c)))
        return c

    def set_config(self, cfg: NwConfig) -> None:
        check(self.lib.nw_set_config(self._h, C.byref(cfg)), "nw_set_config")

    # -- arrays ---------------------------------------------------------------------------
    def _size(self, which: int) -> int:
        if which in (abi.NW_POSITION, abi.NW_VELOCITY):
            return self.n_beads + self.n_solvent
        if which in (abi.NW_TANGENT, abi.NW_FORCE, abi.NW_FORCE_OLD, abi.NW_HASH, abi.NW_SORTED_INDEX):
            return self.n_beads
        if which in (abi.NW_CELL_START, abi.NW_CELL_END):
            return self.n_cells
        if which == abi.NW_SRD_SORTED_INDEX:
            return self.n_beads + self.n_solvent
        return self.n_srd_cells

    def set_array(self, which: int, data, start: int = 0) -> None:
        if which in _FLOAT4:
            a = np.ascontiguousarray(np.asarray(data, dtype=np.float32).reshape(-1, 4))
        else:
            a = np.ascontiguousarray(np.asarray(data, dtype=np.uint32).reshape(-1))
        check(self.lib.nw_set_array(self._h, which, a.ctypes.data, start, a.shape[0]), "nw_set_array")

    def get_array(self, which: int, start: int = 0, count: int | None = None, out: np.ndarray | None = None):
        """Copy `count` elements to host memory (a new array, or `out`, e.g. a
        pinned buffer, which must be C-contiguous with the right dtype)."""
        if count is None:
            count = (out.shape[0] if out is not None else self._size(which) - start)
        if out is None:
            if which in _FLOAT4:
                out = np.empty((count, 4), dtype=np.float32)
            else:
                out = np.empty(count, dtype=np.uint32)
        else:
            want = np.float32 if which in _FLOAT4 else np.uint32
            if out.dtype != want or not out.flags["C_CONTIGUOUS"] or out.shape[0] < count:
                raise ValueError("out must be a C-contiguous array of the array's element type")
        check(self.lib.nw_get_array(self._h, which, out.ctypes.data, start, count), "nw_get_array")
        return out

    def set_array_async(self, which: int, data: np.ndarray, start: int = 0) -> None:
        """nw_set_array_async: enqueue the copy of `data` (kept alive and
        unchanged by the caller until sync(); best pinned) on the stream."""
        want = np.float32 if which in _FLOAT4 else np.uint32
        if data.dtype != want or not data.flags["C_CONTIGUOUS"]:
            raise ValueError("data must be a C-contiguous array of the array's element type")
        n = data.shape[0]
        check(self.lib.nw_set_array_async(self._h, which, data.ctypes.data, start, n), "nw_set_array_async")

    def get_array_async(self, which: int, out: np.ndarray, start: int = 0) -> None:
        """nw_get_array_async: enqueue the copy into `out` (valid after sync())."""
        want = np.float32 if which in _FLOAT4 else np.uint32
        if out.dtype != want or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous array of the array's element type")
        check(self.lib.nw_get_array_async(self._h, which, out.ctypes.data, start, out.shape[0]),
              "nw_get_array_async")

    def device_ptr(self, which: int) -> int:
        p = C.c_void_p()
        check(self.lib.nw_device_array(self._h, which, C.byref(p)), "nw_device_array")
        return p.value or 0

    def zero_forces(self) -> None:
        check(self.lib.nw_zero_forces(self._h), "nw_zero_forces")

    # -- stepping ---------------------------------------------------------------------------
    def step(self, n: int = 1, dt: float = 0.0) -> None:
        check(self.lib.nw_step(self._h, int(n), float(dt)), "nw_step")

    def prepare(self, n: int, dt: float = 0.0, first_step: int | None = None) -> None:
        """Capture the graph that step(n, dt) replays from update first_step
        (default: the current one) without running it."""
        fs = self.step_index if first_step is None else int(first_step)
        check(self.lib.nw_step_prepare(self._h, int(n), float(dt), fs), "nw_step_prepare")

    def sync(self) -> None:
        check(self.lib.nw_sync(self._h), "nw_sync")

    def error_word(self) -> int:
        f = C.c_uint32()
        check(self.lib.nw_error_word(self._h, C.byref(f)))
        return f.value

    @property
    def step_index(self) -> int:
        s = C.c_uint64()
        check(self.lib.nw_get_step(self._h, C.byref(s)))
        return s.value

    def set_step(self, step: int) -> None:
        check(self.lib.nw_set_step(self._h, int(step)))

    def set_graphs(self, enabled: bool) -> None:
        check(self.lib.nw_set_graphs(self._h, 1 if enabled else 0))

    def set_stream(self, stream_handle: int | None) -> None:
        check(self.lib.nw_set_stream(self._h, C.c_void_p(stream_handle or 0)))

    def srd_collide(self, dt_srd: float, shift) -> None:
        s = (C.c_float * 3)(*[float(x) for x in shift])
        check(self.lib.nw_srd_collide(self._h, float(dt_srd), s), "nw_srd_collide")

    @property
    def last_launch_count(self) -> int:
        n = C.c_uint64()
        check(self.lib.nw_last_launch_count(self._h, C.byref(n)))
        return n.value

    def profile(self, n: int, dt: float = 0.0) -> dict:
        """Run n steps with a CUDA event around every kernel; returns
        {kernel name: (total ms, launches)}."""
        buf = (abi.NwKernelTime * 32)()
        cnt = C.c_int()
        check(self.lib.nw_profile_steps(self._h, int(n), float(dt), buf, 32, C.byref(cnt)), "nw_profile_steps")
        return {buf[k].name.decode(): (buf[k].total_ms, int(buf[k].launches)) for k in range(cnt.value)}

    # -- observables (computed on the device) -----------------------------------------------
    def observe(self, min_image: bool = False, msd: bool = False) -> dict:
        """Order parameters, temperatures and (after observe_reset) the mean-
        square displacement of the current state (nw_observe)."""
        o = abi.NwObservables()
        flags = (abi.NW_OBS_MIN_IMAGE if min_image else 0) | (abi.NW_OBS_MSD if msd else 0)
        check(self.lib.nw_observe(self._h, flags, C.byref(o)), "nw_observe")
        return {f: getattr(o, f) for f, _ in o._fields_ if f != "reserved"}

    def observe_reset(self) -> None:
        check(self.lib.nw_observe_reset(self._h), "nw_observe_reset")

    def velocity_correlation(self, i: np.ndarray, j: np.ndarray, r_max: float = 8.0, bins: int = 32):
        """(sum of weighted v_i . v_j, sum of weights) per distance bin of the
        sampled bead pairs (i[k], j[k]) (nw_velocity_correlation)."""
        import torch

        di = torch.from_numpy(np.ascontiguousarray(np.asarray(i, dtype=np.uint32)).view(np.int32)).cuda()
        dj = torch.from_numpy(np.ascontiguousarray(np.asarray(j, dtype=np.uint32)).view(np.int32)).cuda()
        sd = np.zeros(bins, np.float64)
        sw = np.zeros(bins, np.float64)
        torch.cuda.synchronize()
        check(self.lib.nw_velocity_correlation(self._h, di.data_ptr(), dj.data_ptr(), di.numel(), float(r_max), bins,
                                               sd.ctypes.data, sw.ctypes.data), "nw_velocity_correlation")
        return sd, sw

    def srd_temperature_histogram(self, t_max: float, bins: int = 64, shift=(0.0, 0.0, 0.0)) -> np.ndarray:
        """Counts of SRD cells by temperature: bins of t_max / bins, then the
        cells above t_max, then the cells counted (nw_srd_temperature_histogram)."""
        out = np.zeros(bins + 2, np.uint32)
        sh = (C.c_float * 3)(*[float(x) for x in shift])
        check(self.lib.nw_srd_temperature_histogram(self._h, sh, float(t_max), bins, out.ctypes.data),
              "nw_srd_temperature_histogram")
        return out

    def find_defects(self, cell_size: float = 2.0, min_image: bool = False, max_defects: int = 4096) -> np.ndarray:
        """+1/2 and -1/2 defects of the director field of the current beads
        (analysis/find_defects.py:170-207 on the director field of
        analysis/make_director_field.py:10-47, computed on the device).

        Returns a structured array with fields x, y, charge, cells: positive
        defects first, each sign in order of its first grid cell.  cell_size
        is the reference's ``--cellsize`` (default 2); min_image takes bead
        tangents through the periodic boundary (the reference does not)."""
        buf = (abi.NwDefect * max_defects)()
        n = C.c_int()
        flags = abi.NW_DEFECT_MIN_IMAGE if min_image else 0
        check(self.lib.nw_find_defects(self._h, float(cell_size), flags, buf, max_defects, C.byref(n)),
              "nw_find_defects")
        if n.value > max_defects:
            return self.find_defects(cell_size, min_image, n.value)
        return np.frombuffer(buf, dtype=abi.DEFECT_DTYPE, count=n.value).copy()

    def sample_defects(self, beads, radius: float = 10.0, min_image: bool = False) -> np.ndarray:
        """Winding value around the position of each bead in `beads`
        (analysis/defects.py:12-32 on the device); the reference keeps the
        sample points whose value is positive.  `beads` are the sample bead
        indices (the reference draws them with np.random.randint)."""
        idx = np.ascontiguousarray(np.asarray(beads, dtype=np.uint32).reshape(-1))
        out = np.zeros(idx.shape[0], dtype=np.int32)
        flags = abi.NW_DEFECT_MIN_IMAGE if min_image else 0
        check(self.lib.nw_sample_defects(self._h, idx.ctypes.data, int(idx.shape[0]), float(radius), flags,
                                         out.ctypes.data), "nw_sample_defects")
        return out

    # -- checkpoints ------------------------------------------------------------------------
    def checkpoint(self) -> bytes:
        n = C.c_size_t()
        check(self.lib.nw_checkpoint_size(self._h, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        check(self.lib.nw_checkpoint_save(self._h, buf, n.value), "nw_checkpoint_save")
        return buf.raw

    def restore(self, blob: bytes) -> None:
        buf = C.create_string_buffer(blob, len(blob))
        check(self.lib.nw_checkpoint_load(self._h, buf, len(blob)), "nw_checkpoint_load")


class ParticleSystem:
    """Mirror of the reference's ParticleSystem (simulation/particleSystem.h:24-211).

    ``ParticleSystem(numFilaments, filamentSize, gridSize, srdSolvent)`` builds
    the REF_DEM configuration with the reference constructor's defaults;
    setters change the host-side parameters, which are uploaded on the next
    ``update`` (simulation/particleSystem.cpp:255).
    """

    POSITION, VELOCITY, TANGENT = 0, 1, 2

    def __init__(self, numFilaments: int, filamentSize: int, gridSize=(1024, 128, 1), srdSolvent: bool = False,
                 cfg: NwConfig | None = None):
        self._cfg = cfg.copy() if cfg is not None else abi.default_config(
            abi.NW_MODEL_REF_DEM, numFilaments, filamentSize, tuple(gridSize), srdSolvent)
        self._sys = System(self._cfg)
        self._dirty = False
        self._sys.zero_forces()

    # ParticleArray selectors map onto the engine's arrays
    _ARR = {0: abi.NW_POSITION, 1: abi.NW_VELOCITY, 2: abi.NW_TANGENT}

    @property
    def system(self) -> System:
        return self._sys

    def getNumParticles(self) -> int:
        return self._sys.n_beads

    def update(self, deltaTime: float) -> None:
        if self._dirty:
            self._sys.set_config(self._cfg)
            self._dirty = False
        self._sys.step(1, deltaTime)

    def reset(self) -> None:
        """ParticleSystem::reset (simulation/particleSystem.cpp:583-678): the
        reference's lattice state, drawn from rand() after srand(1)."""
        from .init import reference_reset

        pos, vel, tan = reference_reset(self._cfg)
        self._sys.set_array(abi.NW_POSITION, pos)
        self._sys.set_array(abi.NW_VELOCITY, vel)
        self._sys.set_array(abi.NW_TANGENT, tan)
        self._sys.zero_forces()

    def getArray(self, array: int) -> np.ndarray:
        """Bead data (n_beads x 4 floats), like the reference's getArray."""
        return self._sys.get_array(self._ARR[array], 0, self._sys.n_beads)

    def setArray(self, array: int, data, start: int, count: int) -> None:
        a = np.asarray(data, dtype=np.float32).reshape(-1, 4)[:count]
        self._sys.set_array(self._ARR[array], a, start)

    def _set(self, **kw):
        for k, v in kw.items():
            setattr(self._cfg, k, v)
        self._dirty = True

    def setDamping(self, x):
        self._set(gamma=x)

    def setTemperature(self, x):
        self._set(kT=x, srd_kT=x)

    def setGravity(self, x):
        self._cfg.gravity[1] = x
        self._dirty = True

    def setActivity(self, x):
        self._set(activity=x)

    def setReverseProbability(self, x):
        self._set(reverse_probability=x)

    def setCollideSpring(self, x):
        self._set(spring=x)

    def setCollideDamping(self, x):
        self._set(damping=x)

    def setCollideShear(self, x):
        self._set(shear=x)

    def setCollideAttraction(self, x):
        self._set(attraction=x)

    def setBondSpringConstant(self, x):
        self._set(bond_k=x)

    def setBondSpringLength(self, x):
        self._set(bond_r0=x)

    def setBondBendingConstant(self, x):
        self._set(bend_k=x)

    def setBoundaries(self, x, y, z):
        self._cfg.boundary[0], self._cfg.boundary[1], self._cfg.boundary[2] = int(x), int(y), int(z)
        self._dirty = True

    def getParticleRadius(self) -> float:
        return float(self._cfg.radius)

    def getGridSize(self):
        return tuple(int(g) for g in self._cfg.grid)

    def getOrigin(self):
        return tuple(float(o) for o in self._cfg.origin)

    def getCellSize(self):
        return tuple(float(c) for c in self._cfg.cell_size)

    def close(self):
        self._sys.close()
