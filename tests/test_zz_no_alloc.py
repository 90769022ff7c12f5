"""The allocation-free radix sort, pbf_radix_sort_noalloc, through the C ABI.

Some callers cannot allocate device memory while they sort: a host
application whose own allocator has reserved all of the GPU's memory (a
cudaMalloc from the library would fail or take from its pool), or a
real-time loop that must not stall on the allocator.  The variant keeps its scratch in
one device array inside the library (at most 1,048,576 keys), so it must give
exactly what the allocating entry point gives, also on a second call right
after a first one that left the shared array full of another sort's state.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.
"""
import numpy as np
import pytest
import torch

from pbf_gb300 import _capi

pytestmark = pytest.mark.gpu

LIMIT = 1 << 20


def _run(fn, keys: np.ndarray, numbits: int, want_keys: bool = True):
    n = keys.shape[0]
    kin = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    kout = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    perm = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = fn(kin.data_ptr(), kout.data_ptr() if want_keys else None, perm.data_ptr(), n, numbits,
            None)
    _capi.check(st)
    return kout.cpu().numpy().view(np.uint32), perm.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_allocating_sort_on_two_calls(gpu):
    lib = gpu
    rng = np.random.default_rng(2024)
    # first call at the size limit, second smaller with other bits and ties:
    # the second must not see anything the first left in the shared array
    cases = [(LIMIT, 24), (70_001, 19)]
    for n, numbits in cases:
        keys = rng.integers(0, 1 << numbits, n, dtype=np.uint64).astype(np.uint32)
        keys[rng.integers(0, n, n // 4)] = keys[1]
        ka, pa = _run(lib.pbf_radix_sort, keys, numbits)
        kb, pb = _run(lib.pbf_radix_sort_noalloc, keys, numbits)
        # integer work: bit-exact, and a stable argsort
        assert np.array_equal(pb, pa)
        assert np.array_equal(kb, ka)
        assert np.array_equal(pb, np.argsort(keys, kind="stable").astype(np.uint32))


def test_noalloc_sort_without_keys_out(gpu):
    lib = gpu
    keys = (np.arange(5000, dtype=np.uint32) * 2654435761 % 4096).astype(np.uint32)
    _, pa = _run(lib.pbf_radix_sort, keys, 12, want_keys=False)
    _, pb = _run(lib.pbf_radix_sort_noalloc, keys, 12, want_keys=False)
    assert np.array_equal(pb, pa)


def test_noalloc_sort_rejects_more_than_the_limit(gpu):
    lib = gpu
    k = torch.zeros(LIMIT + 1, dtype=torch.int32, device="cuda")
    p = torch.zeros(LIMIT + 1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = lib.pbf_radix_sort_noalloc(k.data_ptr(), None, p.data_ptr(), LIMIT + 1, 8, None)
    assert st == _capi.PBF_ERR_INVALID_ARGUMENT
    assert b"1048576" in lib.pbf_last_error(None)
    assert lib.pbf_radix_sort_noalloc(None, None, None, 0, 8, None) == _capi.PBF_OK
