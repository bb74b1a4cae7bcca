"""The allocation-free radix sort entry point (dbm_radix_sort_pairs_u32_noalloc).

It exists for callers that cannot allocate device memory themselves -- a host program whose own
pool owns all device memory, or a latency-critical loop that cannot take the device-wide
synchronisation of cudaMalloc/cudaFree -- and keeps its scratch in a fixed array inside the
library.  Its output must equal the caller-scratch entry point's (dbm_radix_sort_pairs_u32)
bit for bit, on consecutive calls that reuse the same scratch.

This file is collected last on purpose so that a run stopping at its first failure has already
run every other test; it also passes alone in a fresh process.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_PAIRS = 262144  # DBM_NOALLOC_SORT_MAX_PAIRS in include/direbm_gb300.h


def _lib():
    from direbm_gb300 import _lib

    return _lib.load(), _lib


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _sort_with_caller_scratch(lib, L, keys, vals, bits):
    k = torch.tensor(keys.view(np.int32), device="cuda")
    v = torch.tensor(vals.view(np.int32), device="cuda")
    tmp = torch.empty(int(lib.dbm_radix_sort_tmp_bytes(len(keys), 4)), dtype=torch.uint8, device="cuda")
    L.check(lib.dbm_radix_sort_pairs_u32(k.data_ptr(), v.data_ptr(), len(keys), bits, tmp.data_ptr(), _stream()))
    return k.cpu().numpy().view(np.uint32), v.cpu().numpy().view(np.uint32)


def _sort_noalloc(lib, L, keys, vals, bits):
    k = torch.tensor(keys.view(np.int32), device="cuda")
    v = torch.tensor(vals.view(np.int32), device="cuda")
    L.check(lib.dbm_radix_sort_pairs_u32_noalloc(k.data_ptr(), v.data_ptr(), len(keys), bits, _stream()))
    return k.cpu().numpy().view(np.uint32), v.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_caller_scratch_sort_on_consecutive_calls():
    lib, L = _lib()
    # two calls in a row that share the static scratch: a full-size one, then a smaller one with
    # different data (stale contents of the first call must not leak into the second)
    # 24 and 17 key bits take three 8-bit passes (the result lands in the static alternate buffers
    # and is copied back); 32 and 16 bits take an even number of passes (the result ends in the
    # caller's buffers and the static scratch only ping-pongs); the 32-bit case spans the full key
    # range at the size limit
    for seed, n, bits in ((1, MAX_PAIRS, 24), (2, 100_003, 17), (3, MAX_PAIRS, 32), (4, 65_537, 16)):
        rng = np.random.default_rng(seed)
        keys = rng.integers(0, 1 << bits, size=n, dtype=np.uint64).astype(np.uint32)
        keys[: n // 4] = keys[0]  # long runs of equal keys: the sort must stay stable
        vals = rng.permutation(n).astype(np.uint32)
        k_ref, v_ref = _sort_with_caller_scratch(lib, L, keys, vals, bits)
        k_got, v_got = _sort_noalloc(lib, L, keys, vals, bits)
        np.testing.assert_array_equal(k_got, k_ref)
        np.testing.assert_array_equal(v_got, v_ref)
        order = np.argsort(keys, kind="stable")
        np.testing.assert_array_equal(k_got, keys[order])
        np.testing.assert_array_equal(v_got, vals[order])


def test_noalloc_sort_rejects_sizes_beyond_its_scratch():
    lib, L = _lib()
    n = MAX_PAIRS + 1
    # descending 8-bit keys: any sort that ran would reorder both arrays
    keys = (255 - (np.arange(n, dtype=np.int64) * 256) // n).astype(np.int32)
    k = torch.tensor(keys, device="cuda")
    v = torch.arange(n, dtype=torch.int32, device="cuda")
    rc = lib.dbm_radix_sort_pairs_u32_noalloc(k.data_ptr(), v.data_ptr(), n, 8, _stream())
    assert rc == 3  # DBM_ERR_CAPACITY
    assert b"static scratch limit" in lib.dbm_last_error()
    torch.cuda.synchronize()
    # nothing was queued: keys and values are exactly as they went in
    assert torch.equal(k, torch.tensor(keys, device="cuda"))
    assert torch.equal(v, torch.arange(n, dtype=torch.int32, device="cuda"))
