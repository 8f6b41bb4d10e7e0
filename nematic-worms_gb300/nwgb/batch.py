"""Batched replicas (include/nwgb_batch.h): many WCA worm systems of uneven
size advanced together, one kernel launch per step for all of them."""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import abi
from .abi import NwBatchTuning, NwConfig, check


class Batch:
    """Owns one nw_batch handle.  Replica r's arrays are float4 (n_beads_r, 4)."""

    def __init__(self, configs: Sequence[NwConfig], lib: C.CDLL | None = None):
        self.lib = lib or abi.load_library()
        arr = (NwConfig * len(configs))(*configs)
        h = C.c_void_p()
        check(self.lib.nw_batch_create(arr, len(configs), C.byref(h)), "nw_batch_create")
        self.h = h
        self.configs = list(configs)

    def close(self) -> None:
        if self.h:
            self.lib.nw_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_replicas(self) -> int:
        n = C.c_int()
        t = C.c_uint64()
        check(self.lib.nw_batch_counts(self.h, C.byref(n), C.byref(t)))
        return n.value

    @property
    def total_beads(self) -> int:
        n = C.c_int()
        t = C.c_uint64()
        check(self.lib.nw_batch_counts(self.h, C.byref(n), C.byref(t)))
        return t.value

    def replica(self, r: int):
        nb = C.c_uint32()
        off = C.c_uint64()
        check(self.lib.nw_batch_replica(self.h, r, C.byref(nb), C.byref(off)))
        return nb.value, off.value

    def set_array(self, r: int, which: int, data, start: int = 0) -> None:
        a = np.ascontiguousarray(np.asarray(data, dtype=np.float32).reshape(-1, 4))
        check(self.lib.nw_batch_set_array(self.h, r, which, a.ctypes.data_as(C.c_void_p), start, a.shape[0]),
              "nw_batch_set_array")

    def get_array(self, r: int, which: int) -> np.ndarray:
        nb, _ = self.replica(r)
        out = np.empty((nb, 4), np.float32)
        check(self.lib.nw_batch_get_array(self.h, r, which, out.ctypes.data_as(C.c_void_p), 0, nb),
              "nw_batch_get_array")
        return out

    def step(self, n: int = 1) -> None:
        check(self.lib.nw_batch_step(self.h, n), "nw_batch_step")

    def sync(self) -> None:
        check(self.lib.nw_batch_sync(self.h), "nw_batch_sync")

    def set_graphs(self, on: bool) -> None:
        check(self.lib.nw_batch_set_graphs(self.h, 1 if on else 0))

    def set_stream(self, stream_ptr: int | None) -> None:
        check(self.lib.nw_batch_set_stream(self.h, C.c_void_p(stream_ptr or 0)))

    @property
    def step_index(self) -> int:
        return int(self.lib.nw_batch_get_step(self.h))

    @property
    def last_launch_count(self) -> int:
        v = C.c_uint64()
        check(self.lib.nw_batch_last_launch_count(self.h, C.byref(v)))
        return v.value

    @property
    def tuning(self) -> NwBatchTuning:
        t = NwBatchTuning()
        check(self.lib.nw_batch_get_tuning(self.h, C.byref(t)))
        return t

    def set_tuning(self, threads_per_block: int, strategy: int, neighbor_skin: float,
                   cell_capacity: int = 0) -> None:
        t = NwBatchTuning(threads_per_block, strategy, neighbor_skin, 0.0, cell_capacity)
        check(self.lib.nw_batch_set_tuning(self.h, C.byref(t)), "nw_batch_set_tuning")

    def autotune(self, trial_steps: int = 20) -> NwBatchTuning:
        """Time the candidates and keep the fastest (cached for the batch's
        class); trial_steps = 0 takes the cached tuning of the class."""
        t = NwBatchTuning()
        check(self.lib.nw_batch_autotune(self.h, trial_steps, C.byref(t)), "nw_batch_autotune")
        return t

    @property
    def tuning_class(self) -> tuple[int, int]:
        """(bead-count class, packing class) keying the tuning cache."""
        a, p = C.c_int(), C.c_int()
        check(self.lib.nw_batch_tuning_class(self.h, C.byref(a), C.byref(p)))
        return a.value, p.value
