"""sd_sort_pairs_noalloc: the radix sort for callers that cannot allocate
device memory (for example a stepping loop that must not block on the
device allocator, or a host that only lends this library its own key and
value buffers).  Its scratch is a fixed array inside the library, so the test
checks that two calls in a row -- which share and reuse that array -- give
exactly what sd_sort_pairs gives with a caller-owned scratch buffer, and that
a sort too large for the array is refused.

Kept in a file of its own that pytest collects last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to("cuda:0")


def _host(t):
    return t.cpu().numpy().view(np.uint32)


def sort_with_caller_scratch(sd, keys, vals, key_bits):
    import torch
    k, v = _dev(keys), _dev(vals)
    kt, vt = torch.empty_like(k), torch.empty_like(v)
    nb = sd.SpatialPartition.sort_scratch_bytes(len(keys), key_bits)
    scratch = torch.zeros((nb + 3) // 4, dtype=torch.int32, device="cuda:0")
    sd.SpatialPartition.sort_pairs(k, v, kt, vt, len(keys), key_bits, scratch)
    torch.cuda.synchronize()
    return _host(k), _host(v)


def sort_without_allocation(sd, keys, vals, key_bits):
    import torch
    k, v = _dev(keys), _dev(vals)
    kt, vt = torch.empty_like(k), torch.empty_like(v)
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda:0")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = sd.lib().sd_sort_pairs_noalloc(C.c_void_p(k.data_ptr()), C.c_void_p(v.data_ptr()),
                                        C.c_void_p(kt.data_ptr()), C.c_void_p(vt.data_ptr()), len(keys), key_bits,
                                        C.c_void_p(status.data_ptr()), stream)
    assert rc == 0, sd._abi.last_error()
    torch.cuda.synchronize()
    assert int(status.item()) == 0  # no device error bits
    return _host(k), _host(v)


@pytest.mark.parametrize("key_bits", [18, 25, 32])
def test_noalloc_sort_matches_caller_scratch_sort_twice(sdlib, key_bits):
    rng = np.random.default_rng(key_bits)
    # two calls in a row with different inputs and sizes: the second reuses
    # the array the first left behind
    for n in (1_000_003, 617_001):
        keys = rng.integers(0, 1 << key_bits, n, dtype=np.uint64).astype(np.uint32)
        keys[: n // 4] = keys[0]  # a heavy duplicate run
        vals = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
        ka, va = sort_with_caller_scratch(sdlib, keys, vals, key_bits)
        kb, vb = sort_without_allocation(sdlib, keys, vals, key_bits)
        assert np.array_equal(ka, kb) and np.array_equal(va, vb)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(kb, keys[order]) and np.array_equal(vb, vals[order])


def test_noalloc_sort_rejects_sizes_beyond_its_array(sdlib):
    import torch
    x = torch.zeros(4, dtype=torch.int32, device="cuda:0")
    p = C.c_void_p(x.data_ptr())
    # 2,093,057 keys of 32 bits need more than the 8 MiB array
    rc = sdlib.lib().sd_sort_pairs_noalloc(p, p, p, p, 2_093_057, 32, None, None)
    assert rc == sdlib._abi.SD_ERR_CAPACITY
    assert "scratch" in sdlib._abi.last_error()
