"""nw_sort_particles_noalloc: the stable sort for callers that cannot
allocate device memory (their memory belongs to another allocator, or their
loop cannot take cudaMalloc's implicit synchronisation).  Its scratch is a
fixed array inside the library, shared by every call and keeping the last
call's contents; this checks it sorts exactly like sortParticles on two
calls in a row, and refuses key counts above its 262,144-key limit.

Collected last (file name) so that a run stopping at the first failure has
already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 18


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(t):
    import torch

    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint32)


def _sort_both(lib, keys, vals):
    """Sort the same pairs with sortParticles and with the no-alloc variant."""
    ka, va = _dev(keys.view(np.int32)), _dev(vals.view(np.int32))
    kb, vb = _dev(keys.view(np.int32)), _dev(vals.view(np.int32))
    lib.sortParticles(C.c_void_p(ka.data_ptr()), C.c_void_p(va.data_ptr()), keys.size)
    st = lib.nw_sort_particles_noalloc(C.c_void_p(kb.data_ptr()), C.c_void_p(vb.data_ptr()), keys.size)
    return st, (_host(ka), _host(va)), (_host(kb), _host(vb))


@pytest.mark.parametrize("n,key_range", [(5000, 64), (MAX_KEYS, 1 << 20)])
def test_noalloc_sort_matches_sortParticles_twice(lib, n, key_range):
    rng = np.random.default_rng(n)
    for call in range(2):  # the second call runs on the scratch the first one left behind
        keys = rng.integers(0, key_range, n, dtype=np.uint64).astype(np.uint32)
        vals = np.arange(n, dtype=np.uint32) if call == 0 else rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(
            np.uint32)
        st, (ka, va), (kb, vb) = _sort_both(lib, keys, vals)
        assert st == 0
        assert np.array_equal(ka, kb) and np.array_equal(va, vb)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(kb, keys[order]) and np.array_equal(vb, vals[order])


def test_noalloc_sort_rejects_more_keys_than_its_scratch(lib):
    import torch

    n = MAX_KEYS + 1
    keys = torch.arange(n, 0, -1, dtype=torch.int32, device="cuda")
    vals = torch.zeros(n, dtype=torch.int32, device="cuda")
    st = lib.nw_sort_particles_noalloc(C.c_void_p(keys.data_ptr()), C.c_void_p(vals.data_ptr()), n)
    assert st == 2  # NW_ERR_INVALID
    torch.cuda.synchronize()
    assert int(keys[0].item()) == n  # untouched
