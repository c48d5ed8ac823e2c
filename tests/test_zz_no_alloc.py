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


def _oracle_sort(oracle_mod, keys, vals, offs):
    """libstdc++ std::sort by key of each segment (the oracle), elements past
    the last offset untouched."""
    k, v = keys.copy(), vals.copy()
    for a, b in zip(offs[:-1].astype(np.int64), offs[1:].astype(np.int64)):
        if b > a:
            k[a:b], v[a:b] = oracle_mod.std_sort_u64(k[a:b], v[a:b])
    return k, v


def test_noalloc_sort_matches_libstdcxx_on_partial_ranges_and_mixed_sizes(built_lib,
                                                                          oracle_mod):
    """Against std::sort itself: empty segments, elements after the last
    segment that must stay as they are, and a large call followed by a small
    one and a large one again (the shared scratch keeps the previous call's
    contents)."""
    pytest.importorskip("torch")
    fn = _lib()
    rng = np.random.default_rng(7)
    cases = []
    # large: segments past 4,096 elements take the round-based phase
    sizes = rng.integers(0, 40000, size=40)
    sizes[::5] = 0
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    n = int(offs[-1]) + 5000  # 5,000 trailing elements outside every segment
    cases.append((rng.integers(0, 300, size=n, dtype=np.uint64),
                  rng.integers(0, 1 << 31, size=n, dtype=np.uint32), offs))
    # small: every segment within one block
    sizes = rng.integers(0, 60, size=500)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    n = int(offs[-1]) + 17
    cases.append((rng.integers(0, 8, size=n, dtype=np.uint64),
                  rng.integers(0, 1 << 31, size=n, dtype=np.uint32), offs))
    cases.append(cases[0])
    for keys, vals, offs in cases:
        assert len(keys) <= MAX_ELEMENTS
        got_k, got_v = _noalloc_sort(fn, keys, vals, offs)
        exp_k, exp_v = _oracle_sort(oracle_mod, keys, vals, offs)
        assert np.array_equal(got_k, exp_k)
        assert np.array_equal(got_v, exp_v)
        tail = int(offs[-1])
        assert np.array_equal(got_k[tail:], keys[tail:])
        assert np.array_equal(got_v[tail:], vals[tail:])


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
