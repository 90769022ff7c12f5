"""GPU tests of the standalone stages behind the C ABI: the onesweep radix
sort (RadixSort::Run) and the cell finder (NeighbourCellFinder's findcells),
bit-exact against the oracle / numpy on edge cases."""
import numpy as np
import pytest
import torch

from pbf_gb300 import _capi

pytestmark = pytest.mark.gpu


def gpu_sort(lib, keys, numbits, want_keys=True):
    n = keys.shape[0]
    kin = torch.from_numpy(keys.view(np.int32)).cuda()
    kout = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    perm = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = lib.pbf_radix_sort(kin.data_ptr(), kout.data_ptr() if want_keys else None,
                            perm.data_ptr(), n, numbits, None)
    _capi.check(st)
    return (kout[:n].cpu().numpy().view(np.uint32), perm[:n].cpu().numpy().view(np.uint32))


@pytest.mark.parametrize("n", [1, 2, 31, 4095, 4096, 4097, 65537, 1_000_003])
@pytest.mark.parametrize("numbits", [1, 8, 19, 24, 32])
def test_radix_sort_stable(gpu, oracle_mod, n, numbits):
    rng = np.random.default_rng(n * 131 + numbits)
    hi = 2 ** min(numbits + 2, 32)
    keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    keys[rng.integers(0, n, n // 3 + 1)] = keys[0]  # heavy ties
    ko, po = gpu_sort(gpu, keys, numbits)
    rko, rpo = oracle_mod.radix_sort(keys, numbits)
    assert np.array_equal(po, rpo)
    assert np.array_equal(ko, rko)


@pytest.mark.parametrize("pattern", ["sorted", "reverse", "all_equal", "max_key", "two_values"])
def test_radix_sort_patterns(gpu, oracle_mod, pattern):
    n = 300_001
    if pattern == "sorted":
        keys = np.arange(n, dtype=np.uint32)
    elif pattern == "reverse":
        keys = np.arange(n, dtype=np.uint32)[::-1].copy()
    elif pattern == "all_equal":
        keys = np.full(n, 12345, np.uint32)
    elif pattern == "max_key":
        keys = np.full(n, 0xFFFFFFFF, np.uint32)
        keys[::2] = 0
    else:
        keys = (np.arange(n) % 2).astype(np.uint32)
    ko, po = gpu_sort(gpu, keys, 32, want_keys=(pattern != "two_values"))
    rko, rpo = oracle_mod.radix_sort(keys, 32)
    assert np.array_equal(po, rpo)
    if pattern != "two_values":
        assert np.array_equal(ko, rko)


def test_radix_sort_empty_and_errors(gpu):
    assert gpu.pbf_radix_sort(None, None, None, 0, 8, None) == 0
    k = torch.zeros(8, dtype=torch.int32, device="cuda")
    assert gpu.pbf_radix_sort(k.data_ptr(), None, k.data_ptr(), 8, 8, None) == 1  # aliasing
    p = torch.zeros(8, dtype=torch.int32, device="cuda")
    assert gpu.pbf_radix_sort(k.data_ptr(), None, p.data_ptr(), 8, 0, None) == 1
    assert gpu.pbf_radix_sort(k.data_ptr(), None, p.data_ptr(), 8, 33, None) == 1
    q = torch.zeros(8, dtype=torch.int32, device="cuda")
    # keys_out aliasing perm_out would make the final pass overwrite one with the other
    for fn in (gpu.pbf_radix_sort, gpu.pbf_radix_sort_noalloc):
        assert fn(k.data_ptr(), q.data_ptr(), q.data_ptr(), 8, 8, None) == 1
        assert fn(k.data_ptr(), k.data_ptr(), q.data_ptr(), 8, 8, None) == 1


def ref_cells(sorted_keys, ncells):
    st = np.full(ncells, -1, np.int32)
    en = np.full(ncells, -1, np.int32)
    for i, k in enumerate(sorted_keys):
        if i == 0 or sorted_keys[i - 1] != k:
            st[k] = i
        if i + 1 == len(sorted_keys) or sorted_keys[i + 1] != k:
            en[k] = i + 1
    return st, en


@pytest.mark.parametrize("case", ["single", "first_and_last_cell", "random", "all_one_cell",
                                  "empty"])
def test_find_cells(gpu, case):
    ncells = 1000
    rng = np.random.default_rng(3)
    if case == "single":
        keys = np.array([17], np.uint32)
    elif case == "first_and_last_cell":
        keys = np.array([0, 0, 0, 500, 999, 999], np.uint32)
    elif case == "random":
        keys = np.sort(rng.integers(0, ncells, 20000).astype(np.uint32))
    elif case == "all_one_cell":
        keys = np.full(5000, 3, np.uint32)
    else:
        keys = np.zeros(0, np.uint32)
    n = keys.shape[0]
    kd = torch.from_numpy(keys.view(np.int32).copy() if n else np.zeros(1, np.int32)).cuda()
    st = torch.empty(ncells, dtype=torch.int32, device="cuda")
    en = torch.empty(ncells, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    _capi.check(gpu.pbf_find_cells(kd.data_ptr(), n, ncells, st.data_ptr(), en.data_ptr(), None))
    rst, ren = ref_cells(keys, ncells)
    assert np.array_equal(st.cpu().numpy(), rst)
    assert np.array_equal(en.cpu().numpy(), ren)


def test_find_cells_rejects_key_out_of_range(gpu):
    keys = torch.tensor([1, 2, 50], dtype=torch.int32, device="cuda")
    st = torch.empty(10, dtype=torch.int32, device="cuda")
    en = torch.empty(10, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    assert gpu.pbf_find_cells(keys.data_ptr(), 3, 10, st.data_ptr(), en.data_ptr(), None) == 1


def test_sort_lookback_timeout_is_reported_not_hung(gpu):
    """The onesweep lookback spin is bounded.  pbf_debug_sort_stall makes
    every tile after the first wait on a word nothing sets; each wait gives up
    after the given number of polls, the status word records it and the call
    returns PBF_ERR_DEVICE_FAULT instead of hanging.  The context stays usable:
    the next sort, disarmed, is exact."""
    from pbf_gb300 import _capi
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 1 << 20, 300_000, dtype=np.uint64).astype(np.uint32)  # 74 tiles
    k = torch.from_numpy(keys.view(np.int32)).cuda()
    ko = torch.empty_like(k)
    po = torch.empty_like(k)
    torch.cuda.synchronize()
    try:
        gpu.pbf_debug_sort_stall(1000)
        st = gpu.pbf_radix_sort(k.data_ptr(), ko.data_ptr(), po.data_ptr(), keys.size, 20, None)
    finally:
        gpu.pbf_debug_sort_stall(0)
    assert st == _capi.PBF_ERR_DEVICE_FAULT
    assert b"timed out" in gpu.pbf_last_error(None)
    st = gpu.pbf_radix_sort(k.data_ptr(), ko.data_ptr(), po.data_ptr(), keys.size, 20, None)
    assert st == _capi.PBF_OK
    assert np.array_equal(po.cpu().numpy().view(np.uint32),
                          np.argsort(keys, kind="stable").astype(np.uint32))
