"""The refined reciprocal, square root and quotient of the force laws
against exact (float64, rounded once) results: at most 1 ulp from the
correctly rounded value over positive normal inputs spanning the squared
separations and projections the laws see (1e-4 .. 1e4), checked on the
device through nw_math_probe."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ulps(got: np.ndarray, exact64: np.ndarray) -> np.ndarray:
    want = exact64.astype(np.float32)
    g = got.view(np.int32).astype(np.int64)
    w = want.view(np.int32).astype(np.int64)
    return np.abs(g - w)


def test_refined_helpers_within_one_ulp(lib):
    rng = np.random.default_rng(11)
    n = 1 << 20
    a = np.exp(rng.uniform(np.log(1e-4), np.log(1e4), n)).astype(np.float32)
    b = np.exp(rng.uniform(np.log(1e-4), np.log(1e4), n)).astype(np.float32)
    out = np.empty((n, 4), np.float32)
    st = lib.nw_math_probe(a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p), n,
                           out.ctypes.data_as(C.c_void_p))
    assert st == 0
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    assert ulps(out[:, 0], 1.0 / a64).max() <= 1
    assert ulps(out[:, 1], np.sqrt(a64)).max() <= 1
    assert ulps(out[:, 2], a64 / b64).max() <= 1
    # the hardware reciprocal square root stays inside its documented 2 ulp
    assert ulps(out[:, 3], 1.0 / np.sqrt(a64)).max() <= 2
