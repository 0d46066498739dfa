"""Reference-compatible spatial hash on the GPU (SpatialPartition operators)
against the CPU oracle: construct (keys, sphere words, count), sort, and
candidate pairs are bit-exact, in the reference's traversal order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gpu_pipeline(sd, pos, sizes, cell, body_of=None, cap=None):
    import torch
    dev = torch.device("cuda:0")
    n = len(pos)
    P = sd.SpatialPartition
    tpos = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).to(dev)
    tsz = torch.from_numpy(np.ascontiguousarray(sizes, np.float32)).to(dev)
    cells = torch.empty(9 * n, dtype=torch.int32, device=dev)
    spheres = torch.empty(9 * n, dtype=torch.int32, device=dev)
    count = torch.zeros(1, dtype=torch.int32, device=dev)
    P.construct_collision_list(n, cell, cells, spheres, tsz, tpos, count)
    built = (cells.cpu().numpy().view(np.uint32).copy(), spheres.cpu().numpy().view(np.uint32).copy(),
             int(count.item()))
    ct = torch.empty_like(cells)
    st = torch.empty_like(spheres)
    nb = P.sort_scratch_bytes(9 * n, 32)
    scratch = torch.zeros((nb + 3) // 4, dtype=torch.int32, device=dev)
    P.sort_collision_list(cells, spheres, ct, st, 9 * n, scratch)
    assert P.sort_status(scratch) == 0
    sorted_ = (cells.cpu().numpy().view(np.uint32).copy(), spheres.cpu().numpy().view(np.uint32).copy())
    cap = cap if cap is not None else 40 * n + 16
    pa = torch.empty(cap, dtype=torch.int32, device=dev)
    pb = torch.empty(cap, dtype=torch.int32, device=dev)
    npairs = torch.zeros(1, dtype=torch.int64, device=dev)
    ps = torch.zeros((P.pairs_scratch_bytes(9 * n) + 3) // 4, dtype=torch.int32, device=dev)
    bo = None if body_of is None else torch.from_numpy(np.ascontiguousarray(body_of, np.int32)).to(dev)
    P.candidate_pairs(cells, spheres, count, 9 * n, bo, pa, pb, cap, npairs, ps)
    torch.cuda.synchronize()
    m = int(npairs.item())
    k = min(m, cap)
    pairs = (pa[:k].cpu().numpy().view(np.uint32), pb[:k].cpu().numpy().view(np.uint32), m)
    return built, sorted_, pairs


@pytest.mark.parametrize("n,cell,size", [(1, 0.25, 0.1), (1000, 1 / 16, 0.03), (50_000, 1 / 64, 0.008),
                                         (300_000, 1 / 128, 0.004)])
def test_hash_pipeline_bit_exact(sdlib, orc, n, cell, size):
    rng = np.random.default_rng(n)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0, 1, (n, 3))
    sizes = np.full(n, size, np.float32)
    built, sorted_, pairs = gpu_pipeline(sdlib, pos, sizes, cell)
    oc, osp, ocount = orc.ref_hash_build(pos, sizes, cell)
    assert built[2] == ocount
    assert np.array_equal(built[0], oc) and np.array_equal(built[1], osp)
    ko, vo = orc.radix_sort_pairs(oc, osp, 32)
    assert np.array_equal(sorted_[0], ko) and np.array_equal(sorted_[1], vo)
    a, b = orc.ref_candidate_pairs(ko, vo, ocount)
    assert pairs[2] == len(a)
    assert np.array_equal(pairs[0], a) and np.array_equal(pairs[1], b)


def test_hash_edge_positions(sdlib, orc):
    """Cell-boundary, domain-edge, out-of-domain and polydisperse inputs."""
    cell = 1.0 / 8
    vals = np.array([0.0, cell, 2 * cell, 1 - 1e-7, 0.999, 1.0, 1.5, -0.0, 0.0625, 0.1249999], np.float32)
    g = np.stack(np.meshgrid(vals, vals, vals, indexing="ij"), -1).reshape(-1, 3)
    pos = np.zeros((len(g), 4), np.float32)
    pos[:, :3] = g
    sizes = np.random.default_rng(0).uniform(0.0, 0.2, len(g)).astype(np.float32)
    built, sorted_, pairs = gpu_pipeline(sdlib, pos, sizes, cell)
    oc, osp, ocount = orc.ref_hash_build(pos, sizes, cell)
    assert built[2] == ocount
    assert np.array_equal(built[0], oc) and np.array_equal(built[1], osp)
    ko, vo = orc.radix_sort_pairs(oc, osp, 32)
    assert np.array_equal(sorted_[0], ko) and np.array_equal(sorted_[1], vo)


def test_candidate_pairs_skip_same_body(sdlib, orc):
    rng = np.random.default_rng(9)
    n = 20_000
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0, 1, (n, 3))
    sizes = np.full(n, 0.02, np.float32)
    body = (np.arange(n) // 4).astype(np.int32)
    _, _, pairs = gpu_pipeline(sdlib, pos, sizes, 1 / 32, body_of=body)
    oc, osp, ocount = orc.ref_hash_build(pos, sizes, 1 / 32)
    ko, vo = orc.radix_sort_pairs(oc, osp, 32)
    a, b = orc.ref_candidate_pairs(ko, vo, ocount, body)
    assert np.array_equal(pairs[0], a) and np.array_equal(pairs[1], b)


def test_candidate_pairs_overflow_counts_all(sdlib, orc):
    rng = np.random.default_rng(10)
    n = 5000
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0, 1, (n, 3))
    sizes = np.full(n, 0.03, np.float32)
    _, _, pairs = gpu_pipeline(sdlib, pos, sizes, 1 / 16, cap=100)
    oc, osp, ocount = orc.ref_hash_build(pos, sizes, 1 / 16)
    ko, vo = orc.radix_sort_pairs(oc, osp, 32)
    a, b = orc.ref_candidate_pairs(ko, vo, ocount)
    assert pairs[2] == len(a) > 100
    assert np.array_equal(pairs[0], a[:100]) and np.array_equal(pairs[1], b[:100])
