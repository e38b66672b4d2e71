"""Allocation-free radix sort (scratch in a fixed device array of the library) against the
allocating entry point ndt_radix_sort_pairs_u64_u32, through the C ABI.

The two must agree bit for bit (integer sort). Each case calls the allocation-free entry
twice in a row on fresh copies of the input, so the second call runs on scratch the first
one left behind. This file is collected last so that it also runs after every other test
has used the library in the same process."""
import ctypes as C

import numpy as np
import pytest

from cuda_ndt_matcher_gb300 import capi

pytestmark = pytest.mark.gpu

MAX_PAIRS = 1 << 20
NDT_ERR_CAPACITY = -10


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _device_pair(torch, keys, vals):
    k = torch.from_numpy(np.asarray(keys, np.uint64).view(np.int64).copy()).cuda()
    v = torch.from_numpy(np.asarray(vals, np.uint32).view(np.int32).copy()).cuda()
    return k, v


def _host(torch, k, v):
    torch.cuda.synchronize()
    return k.cpu().numpy().view(np.uint64), v.cpu().numpy().view(np.uint32)


def sort_allocating(torch, keys, vals, begin, end):
    L = capi.load()
    k, v = _device_pair(torch, keys, vals)
    tb = C.c_uint64(0)
    capi.check(L.ndt_radix_sort_pairs_u64_u32(_ptr(k), _ptr(v), len(keys), begin, end, None,
                                              C.byref(tb), None))
    tmp = torch.empty(max(int(tb.value), 1), dtype=torch.uint8, device="cuda")
    capi.check(L.ndt_radix_sort_pairs_u64_u32(_ptr(k), _ptr(v), len(keys), begin, end,
                                              _ptr(tmp), C.byref(tb), None))
    return _host(torch, k, v)


def sort_static(torch, keys, vals, begin, end):
    L = capi.load()
    k, v = _device_pair(torch, keys, vals)
    capi.check(L.ndt_radix_sort_pairs_u64_u32_static(_ptr(k), _ptr(v), len(keys), begin, end,
                                                     None))
    return _host(torch, k, v)


@pytest.mark.parametrize("n,begin,end", [(1, 0, 64), (4097, 0, 64), (100_003, 0, 64),
                                         (250_000, 8, 40), (MAX_PAIRS, 0, 64)])
def test_static_sort_matches_allocating(gpu, n, begin, end):
    import torch
    rng = np.random.default_rng(n + begin)
    keys = rng.integers(0, 2 ** 64 - 1, n, dtype=np.uint64)
    keys[::7] = keys[0]            # many equal keys: exercises stability
    vals = np.arange(n, dtype=np.uint32)
    ref_k, ref_v = sort_allocating(torch, keys, vals, begin, end)
    for _ in range(2):
        k, v = sort_static(torch, keys, vals, begin, end)
        assert np.array_equal(k, ref_k)
        assert np.array_equal(v, ref_v)
    if begin == 0 and end == 64:
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(ref_v, vals[order])


def test_static_sort_rejects_oversize(gpu):
    import torch
    L = capi.load()
    k = torch.zeros(4, dtype=torch.int64, device="cuda")
    v = torch.zeros(4, dtype=torch.int32, device="cuda")
    rc = L.ndt_radix_sort_pairs_u64_u32_static(_ptr(k), _ptr(v), MAX_PAIRS + 1, 0, 64, None)
    assert rc == NDT_ERR_CAPACITY
    assert b"1048576" in L.ndt_last_error_string()
    torch.cuda.synchronize()
    assert int(k.abs().sum().item()) == 0
