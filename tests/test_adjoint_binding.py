"""Host-side checks of the adjoint binding without a GPU: the handle rejects
what it does not support before touching a device."""
from __future__ import annotations

import ctypes as C

from nwgb import abi
from nwgb.init import wca_config


def test_create_rejects_unsupported_configurations(lib):
    h = C.c_void_p()
    c = wca_config(10, 10, (20.0, 20.0), srd=True, lib=lib)
    assert lib.nw_adj_create(C.byref(c), 1, 10, 5, 32, C.byref(h)) == abi.NW_ERR_UNSUPPORTED
    c = wca_config(10, 10, (20.0, 20.0), lib=lib)
    assert lib.nw_adj_create(C.byref(c), 1, 10, 5, 16, C.byref(h)) == abi.NW_ERR_INVALID
    assert lib.nw_adj_create(C.byref(c), 0, 10, 5, 32, C.byref(h)) == abi.NW_ERR_INVALID
    c.boundary[0] = abi.NW_WALL
    assert lib.nw_adj_create(C.byref(c), 1, 10, 5, 32, C.byref(h)) == abi.NW_ERR_UNSUPPORTED
