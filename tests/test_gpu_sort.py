"""Onesweep radix sort (sd_sort_pairs) against a stable CPU sort: bit-exact
keys and values for every key width, duplicate-heavy and ragged inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run_sort(sd, keys, vals, key_bits):
    import torch
    n = len(keys)
    dev = torch.device("cuda:0")
    k = torch.from_numpy(keys.view(np.int32)).to(dev)
    v = torch.from_numpy(vals.view(np.int32)).to(dev)
    kt = torch.empty_like(k)
    vt = torch.empty_like(v)
    nb = sd.SpatialPartition.sort_scratch_bytes(n, key_bits)
    scratch = torch.zeros((nb + 3) // 4, dtype=torch.int32, device=dev)
    sd.SpatialPartition.sort_pairs(k, v, kt, vt, n, key_bits, scratch)
    assert sd.SpatialPartition.sort_status(scratch) == 0
    torch.cuda.synchronize()
    return k.cpu().numpy().view(np.uint32), v.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("n", [1, 2, 31, 2047, 2048, 2049, 100_000, 1_000_003])
@pytest.mark.parametrize("key_bits", [18, 20, 32])
def test_sort_random(sdlib, n, key_bits):
    rng = np.random.default_rng(n + key_bits)
    keys = rng.integers(0, 1 << key_bits, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    k, v = run_sort(sdlib, keys, vals, key_bits)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order])
    assert np.array_equal(v, vals[order])


@pytest.mark.parametrize("key_bits", [1, 5, 8, 9, 10, 17, 19, 20, 21, 25, 27])
def test_sort_key_widths(sdlib, key_bits):
    rng = np.random.default_rng(key_bits)
    n = 300_000
    keys = rng.integers(0, 1 << key_bits, n, dtype=np.uint64).astype(np.uint32)
    vals = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    k, v = run_sort(sdlib, keys, vals, key_bits)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order]) and np.array_equal(v, vals[order])


@pytest.mark.parametrize("kind", ["all_equal", "two_values", "sorted", "reversed", "max_values", "few_runs"])
def test_sort_adversarial(sdlib, kind):
    n = 500_000
    rng = np.random.default_rng(1)
    if kind == "all_equal":
        keys = np.full(n, 12345, np.uint32)
    elif kind == "two_values":
        keys = rng.integers(0, 2, n).astype(np.uint32) * np.uint32(0xFFFF0000)
    elif kind == "sorted":
        keys = np.sort(rng.integers(0, 1 << 32, n, dtype=np.uint64)).astype(np.uint32)
    elif kind == "reversed":
        keys = np.sort(rng.integers(0, 1 << 32, n, dtype=np.uint64))[::-1].astype(np.uint32)
    elif kind == "max_values":
        keys = np.full(n, 0xFFFFFFFF, np.uint32)
        keys[::7] = 0
    else:
        keys = np.repeat(rng.integers(0, 1 << 32, 50, dtype=np.uint64).astype(np.uint32), n // 50)
    vals = np.arange(len(keys), dtype=np.uint32)
    k, v = run_sort(sdlib, keys, vals, 32)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order]) and np.array_equal(v, vals[order])


def test_sort_matches_oracle_on_hash_entries(sdlib, orc):
    """9n reference-layout entries of 200k spheres (1.8M pairs) sorted by the
    full cell word: identical to the oracle's stable LSD sort."""
    rng = np.random.default_rng(3)
    n = 200_000
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0, 1, (n, 3))
    sizes = np.full(n, 0.004, np.float32)
    cells, spheres, count = orc.ref_hash_build(pos, sizes, 1.0 / 128)
    k, v = run_sort(sdlib, cells, spheres, 32)
    ko, vo = orc.radix_sort_pairs(cells, spheres, 32)
    assert np.array_equal(k, ko) and np.array_equal(v, vo)


def test_sort_empty_and_bad_args(sdlib):
    import ctypes as C
    import torch
    st = sdlib.lib().sd_sort_pairs(None, None, None, None, 0, 32, None, 0, None)
    assert st == 0
    x = torch.zeros(16, dtype=torch.int32, device="cuda")
    st = sdlib.lib().sd_sort_pairs(C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()),
                                   C.c_void_p(x.data_ptr()), 16, 32, C.c_void_p(x.data_ptr()), 64, None)
    assert st == sdlib._abi.SD_ERR_CAPACITY  # scratch too small
    st = sdlib.lib().sd_sort_pairs(None, None, None, None, 16, 33, None, 0, None)
    assert st == sdlib._abi.SD_ERR_INVALID_ARG
