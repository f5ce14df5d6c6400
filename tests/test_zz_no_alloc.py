"""snch_sort_pairs_noalloc -- the sort for callers that cannot allocate GPU memory
(a solver loop that must not stall the device on cudaMalloc/cudaFree, a plug-in
whose GPU memory belongs to its host application) -- against the allocating
snch_sort_pairs, through the C ABI.

Sorting is exact, so outputs must be identical. Two calls in a row with
different data and sizes check that the shared working array carries nothing
over from one call to the next. Collected last (file name) so that a run that
stops at the first failure has run every other test first; it also passes
alone in a fresh process.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def max_pairs():
    text = open(os.path.join(ROOT, "include", "snch_gb300.h")).read()
    return int(re.search(r"#define SNCH_SORT_NOALLOC_MAX_PAIRS (\d+)", text).group(1))


def ptr(t):
    return C.c_void_p(t.data_ptr())


def sort_existing(L, keys, vals, bits, stream):
    import torch
    n = keys.numel()
    k, v = keys.clone(), vals.clone()
    kt, vt = torch.empty_like(k), torch.empty_like(v)
    scratch = torch.empty(L.snch_sort_scratch_bytes(n, bits), dtype=torch.uint8, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.snch_sort_pairs(ptr(k), ptr(v), ptr(kt), ptr(vt), n, bits, ptr(scratch), ptr(status), stream)
    assert rc == 0, L.snch_last_error()
    return k, v, status


def sort_noalloc(L, keys, vals, bits, stream):
    import torch
    ko, vo = torch.empty_like(keys), torch.empty_like(vals)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.snch_sort_pairs_noalloc(ptr(keys), ptr(vals), ptr(ko), ptr(vo), keys.numel(), bits, ptr(status), stream)
    assert rc == 0, L.snch_last_error()
    return ko, vo, status


def test_noalloc_sort_matches_allocating_sort_twice():
    import torch
    assert torch.cuda.is_available()
    from snch_lbvh_gb300 import _ffi
    L = _ffi.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(7)
    cases = [
        (1_000_000, 30, rng.integers(0, 1 << 12, 1_000_000, dtype=np.uint32) << np.uint32(18)),  # many duplicates
        (max_pairs(), 32, rng.integers(0, 1 << 32, max_pairs(), dtype=np.uint64).astype(np.uint32)),
        (4097, 24, rng.integers(0, 1 << 24, 4097, dtype=np.uint32)),  # odd pass count, ragged tile
    ]
    for n, bits, keys_np in cases:
        keys = torch.from_numpy(keys_np.view(np.int32)).cuda()
        vals = torch.from_numpy(rng.permutation(n).astype(np.int32)).cuda()
        ek, ev, es = sort_existing(L, keys, vals, bits, stream)
        nk, nv, ns = sort_noalloc(L, keys, vals, bits, stream)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(nk.cpu().numpy(), ek.cpu().numpy())
        np.testing.assert_array_equal(nv.cpu().numpy(), ev.cpu().numpy())
        assert int(es.item()) == 0 and int(ns.item()) == 0
        # and both are the stable sort of the input
        order = np.argsort(keys_np & np.uint32((1 << bits) - 1 if bits < 32 else 0xFFFFFFFF), kind="stable")
        np.testing.assert_array_equal(nv.cpu().numpy(), vals.cpu().numpy()[order])


def test_noalloc_sort_in_place_and_without_status_word():
    """keys_out == keys_in and values_out == values_in (documented as allowed),
    and device_status NULL (the bits then go to the shared array's own word),
    each against snch_sort_pairs, twice in a row."""
    import torch
    from snch_lbvh_gb300 import _ffi
    L = _ffi.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(11)
    for n, bits in ((300_001, 30), (65_536, 32)):
        keys_np = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
        keys = torch.from_numpy(keys_np.view(np.int32)).cuda()
        vals = torch.from_numpy(rng.permutation(n).astype(np.int32)).cuda()
        ek, ev, _ = sort_existing(L, keys, vals, bits, stream)
        k, v = keys.clone(), vals.clone()
        rc = L.snch_sort_pairs_noalloc(ptr(k), ptr(v), ptr(k), ptr(v), n, bits, None, stream)
        assert rc == 0, L.snch_last_error()
        ko, vo = torch.empty_like(keys), torch.empty_like(vals)
        rc = L.snch_sort_pairs_noalloc(ptr(keys), ptr(vals), ptr(ko), ptr(vo), n, bits, None, stream)
        assert rc == 0, L.snch_last_error()
        torch.cuda.synchronize()
        for a, b in ((k, ek), (v, ev), (ko, ek), (vo, ev)):
            np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())


def test_noalloc_sort_rejects_sizes_beyond_its_limit():
    import torch
    from snch_lbvh_gb300 import _ffi
    L = _ffi.lib()
    n = max_pairs() + 1
    rc = L.snch_sort_pairs_noalloc(None, None, None, None, n, 30, None, None)
    assert rc == 6  # SNCH_ERR_TOO_LARGE, before touching the GPU
    assert str(max_pairs()) in L.snch_last_error().decode()
    assert L.snch_sort_pairs_noalloc(None, None, None, None, 10, 33, None, None) == 1
    torch.cuda.synchronize()
