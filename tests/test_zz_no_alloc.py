"""The allocation-free sort entry point, for callers that may not allocate
device memory (their GPU memory belongs to another allocator, or their
footprint is fixed in advance).  Through the C ABI it must give exactly the
result of the ordinary entry point, call after call, while using only its
fixed scratch array.  This file is collected last on purpose."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ELEMENTS = 1048576
MAX_SEGMENTS = 65536


def _lib():
    from cuflye_gb300.backend import load_library
    L = load_library()
    f = L.cuflye_std_sort_segments_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                  ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p]
    return f


def _case(seed, n_segments, max_len, key_range):
    rng = np.random.default_rng(seed)
    sizes = rng.integers(0, max_len, size=n_segments)
    sizes[::11] = rng.integers(5000, 30000, size=len(sizes[::11]))  # large segments too
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    n = int(offs[-1])
    keys = rng.integers(0, key_range, size=n, dtype=np.uint64)
    vals = rng.integers(0, 1 << 31, size=n, dtype=np.uint32)
    return keys, vals, offs


def _noalloc_sort(fn, keys, vals, offs):
    import torch
    dk = torch.from_numpy(keys.view(np.int64).copy()).cuda()
    dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    torch.cuda.synchronize()
    o = np.ascontiguousarray(offs, dtype=np.uint64)
    st = fn(ctypes.c_void_p(dk.data_ptr()), ctypes.c_void_p(dv.data_ptr()),
            o.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), len(o) - 1, len(keys), None)
    assert st == 0
    torch.cuda.synchronize()
    return dk.cpu().numpy().view(np.uint64), dv.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_std_sort_entry_point_twice(built_lib):
    torch = pytest.importorskip("torch")
    from cuflye_gb300.backend import CudaBackend
    fn = _lib()
    with CudaBackend(device=0, memory_budget_bytes=0) as ref:
        for seed, nseg, maxlen, kr in ((1, 300, 3000, 64), (2, 120, 9000, 1 << 40)):
            keys, vals, offs = _case(seed, nseg, maxlen, kr)
            assert len(keys) <= MAX_ELEMENTS
            got_k, got_v = _noalloc_sort(fn, keys, vals, offs)
            exp_k, exp_v = ref.std_sort_segments(keys, vals, offs)
            assert np.array_equal(got_k, exp_k)
            assert np.array_equal(got_v, exp_v)


def test_noalloc_rejects_oversized_requests(built_lib):
    pytest.importorskip("torch")
    fn = _lib()
    offs = np.array([0, 10], dtype=np.uint64)
    # larger than the fixed scratch: refused before anything is queued
    st = fn(ctypes.c_void_p(0), ctypes.c_void_p(0),
            offs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), 1, MAX_ELEMENTS + 1, None)
    assert st == 2  # CUFLYE_ERR_UNSUPPORTED
    many = np.zeros(MAX_SEGMENTS + 2, dtype=np.uint64)
    st = fn(ctypes.c_void_p(0), ctypes.c_void_p(0),
            many.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), MAX_SEGMENTS + 1, 0, None)
    assert st == 2
