"""The allocation-free sort entry point (bh_sort_keys_noalloc).

It exists for callers that cannot let the engine call cudaMalloc -- a host
code whose device memory belongs to its own pool, or a time-critical loop that
cannot take cudaMalloc's implicit synchronisation -- and keeps its scratch in
a fixed device array shared by all calls.  These checks call it through the C
ABI on device buffers the test owns and compare it with the existing sort
entry point (bh_sort_bodies_by_morton_key), on several calls in a row, so that
contents left in the shared scratch by one call cannot leak into the next.

This file is collected last on purpose: a run that stops at the first failure
has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry(bh):
    lib = bh.library()
    fn = lib.bh_sort_keys_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    return lib, fn


def _existing_sort(bh, keys):
    """Sorted keys and permutation from the existing entry point."""
    n = len(keys)
    ids = np.arange(n, dtype=np.uint64)
    zeros3 = np.zeros((n, 3))
    sk, _, _, _, si = bh.sortBodiesByMortonKey(keys, zeros3, np.zeros(n), zeros3, ids)
    return sk, si.astype(np.int64)


def _noalloc_sort(fn, keys, in_place=False):
    """Calls the entry point on device copies of `keys`; with in_place the
    same buffer is passed as keys_in and keys_out."""
    import torch
    n = len(keys)
    d_in = torch.from_numpy(np.ascontiguousarray(keys).view(np.int64).copy()).cuda()
    d_out = d_in if in_place else torch.full_like(d_in, -1)
    d_perm = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = fn(d_in.data_ptr(), d_out.data_ptr(), d_perm.data_ptr(), n, None)
    return rc, d_out.cpu().numpy().view(np.uint64)[:n], d_perm.cpu().numpy().astype(np.int64)[:n]


def _stable_sort(keys):
    """An independent stable sort: numpy's, on the unsigned keys."""
    perm = np.argsort(keys, kind="stable")
    return keys[perm], perm.astype(np.int64)


def test_noalloc_sort_matches_existing_entry_point_on_consecutive_calls(bh):
    lib, fn = _entry(bh)
    cases = []
    pos, _, _, _ = bh.generate_system(2, 300_149, 0.1, 0.0)
    cases.append(bh.generateMortonCodes(pos, bh.compute_local_bbox(pos)))
    pos, _, _, _ = bh.generate_system(7, 1_000, 0.1, 0.05)
    cases.append(bh.generateMortonCodes(pos, bh.compute_local_bbox(pos)))
    rng = np.random.default_rng(3)
    dup = rng.integers(0, 1 << 63, 70_000, dtype=np.uint64)
    dup[rng.integers(0, 70_000, 5_000)] = dup[:5_000]  # repeated keys: the order of ties must match too
    cases.append(dup)
    cases.append(cases[1].copy())  # the small case again, after the larger ones
    for keys in cases:
        ref_keys, ref_perm = _existing_sort(bh, keys)
        rc, got_keys, got_perm = _noalloc_sort(fn, keys)
        assert rc == 0, lib.bh_last_error()
        assert np.array_equal(got_keys, ref_keys)
        assert np.array_equal(got_perm, ref_perm)
        want_keys, want_perm = _stable_sort(keys)
        assert np.array_equal(got_keys, want_keys) and np.array_equal(got_perm, want_perm)


def test_noalloc_sort_in_place_single_key_and_top_bit(bh):
    """keys_in == keys_out (the header allows it), twice in a row; a single
    key in place and not; keys with bit 63 set among ties and small values
    (the eight digit passes cover all 64 bits); each against numpy's stable
    sort."""
    lib, fn = _entry(bh)
    rng = np.random.default_rng(9)
    big = rng.integers(0, 1 << 63, 200_000, dtype=np.uint64) | (rng.integers(0, 2, 200_000, dtype=np.uint64) << 63)
    big[rng.integers(0, 200_000, 20_000)] = big[:20_000]
    big[:7] = [np.uint64(0xFFFFFFFFFFFFFFFF), 0, np.uint64(1 << 63), 0, np.uint64(0xFFFFFFFFFFFFFFFF), 1,
               np.uint64(1 << 63)]
    for keys, in_place in ((big, True), (big, True), (big[:1], True), (big[:1], False), (big[:2], True),
                           (big[:4096 * 3 + 5], False)):
        rc, got_keys, got_perm = _noalloc_sort(fn, keys, in_place=in_place)
        assert rc == 0, lib.bh_last_error()
        want_keys, want_perm = _stable_sort(keys)
        assert np.array_equal(got_keys, want_keys), (len(keys), in_place)
        assert np.array_equal(got_perm, want_perm), (len(keys), in_place)


def test_noalloc_sort_rejects_sizes_beyond_its_scratch(bh):
    import torch
    lib, fn = _entry(bh)
    limit = 1 << 20
    d = torch.zeros(8, dtype=torch.int64, device="cuda")
    rc = fn(d.data_ptr(), d.data_ptr(), d.data_ptr(), limit + 1, None)
    assert rc == 4  # BH_ERR_CAPACITY
    assert str(limit).encode() in lib.bh_last_error()
    assert fn(d.data_ptr(), d.data_ptr(), d.data_ptr(), 0, None) == 0
