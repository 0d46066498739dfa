"""Sweep and prune on the GPU: the reference's windowed sweep rows against
the reference kernel's own output (tests/golden/ref_sap_*.npz) and the
oracle, and the exact pair operator against the oracle's pair sets."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("case", ["a", "b"])
def test_sap_sweep_matches_reference_kernel(sdlib, case):
    import torch
    g = np.load(GOLDEN / f"ref_sap_{case}.npz")
    t = lambda k: torch.from_numpy(np.ascontiguousarray(g[k])).cuda()
    rows = sdlib.SweepAndPrune.sweep(t("upperx"), t("lowerx_sorted"), t("uppery"), t("lowery"), t("idx_sorted"))
    assert np.array_equal(rows.cpu().numpy(), g["rows"])
    rows2 = sdlib.SweepAndPrune.process_collisions(t("pos"))
    assert np.array_equal(rows2.cpu().numpy(), g["rows"])


@pytest.mark.parametrize("n,seed", [(0, 0), (1, 0), (2, 1), (5000, 2), (200_000, 3)])
def test_sap_process_matches_oracle(sdlib, orc, n, seed):
    import torch
    rng = np.random.default_rng(seed)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0.0, 1.0, (n, 3))
    pos[:, 3] = rng.uniform(0.001, 0.01, n)
    rows = sdlib.SweepAndPrune.process_collisions(torch.from_numpy(pos).cuda())
    assert np.array_equal(rows.cpu().numpy(), orc.sap_process(pos))


@pytest.mark.parametrize("n,seed", [(0, 0), (1, 0), (2, 1), (3000, 4), (100_000, 5)])
def test_sap_pairs_bit_exact(sdlib, orc, n, seed):
    import torch
    rng = np.random.default_rng(seed)
    c = rng.uniform(-0.4, 1.6, (n, 3)).astype(np.float32)
    h = rng.uniform(0.001, 0.015, (n, 3)).astype(np.float32)
    L = np.zeros((n, 4), np.float32)
    H = np.zeros((n, 4), np.float32)
    L[:, :3] = c - h
    H[:, :3] = c + h
    if n >= 2:
        L[1], H[1] = L[0], H[0]
    want = orc.aabb_pairs(L, H)
    got, cnt, err = sdlib.SweepAndPrune.pairs(torch.from_numpy(L).cuda(), torch.from_numpy(H).cuda(), len(want) + 8)
    assert err == 0 and cnt == len(want)
    assert np.array_equal(got.cpu().numpy().view(np.uint64), want)


def test_sap_pairs_overflow_is_reported(sdlib):
    import torch
    rng = np.random.default_rng(9)
    c = rng.uniform(0, 1, (2000, 3)).astype(np.float32)
    L = np.zeros((2000, 4), np.float32)
    H = np.zeros((2000, 4), np.float32)
    L[:, :3] = c - 0.05
    H[:, :3] = c + 0.05
    got, cnt, err = sdlib.SweepAndPrune.pairs(torch.from_numpy(L).cuda(), torch.from_numpy(H).cuda(), 10)
    assert err & sdlib._abi.SD_DEVERR_PAIR_OVERFLOW


def _scene(kind, n, seed):
    """Boxes that stress the binned sweep's column grid: mixed sizes with a
    few boxes spanning the domain, corners on column boundaries, a flat
    scene (no y-z extent at all), y/z-inverted boxes, large coordinates."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-0.7, 1.3, (n, 3)).astype(np.float32)
    h = np.exp(rng.normal(np.log(0.006), 0.6, (n, 3))).astype(np.float32)
    if kind == "mixed":
        h[rng.random(n) < 0.01] = 0.0
        big = rng.random(n) < 0.002
        h[big] = rng.uniform(0.2, 0.9, (int(big.sum()), 3))
    elif kind == "aligned":
        c = (rng.integers(0, 96, (n, 3)) / 64.0).astype(np.float32)
        h = (rng.integers(0, 3, (n, 3)) / 128.0).astype(np.float32)
    elif kind == "flat":
        c[:, 1:] = 0.5
        h[:, 1:] = 0.0
    elif kind == "large":
        c = (c * 1000.0 + 1.0e6).astype(np.float32)
        h = (h * 1000.0).astype(np.float32)
    L = np.zeros((n, 4), np.float32)
    H = np.zeros((n, 4), np.float32)
    L[:, :3] = c - h
    H[:, :3] = c + h
    if kind == "inverted_yz":
        flip = rng.random(n) < 0.1
        L[flip, 1], H[flip, 1] = H[flip, 1].copy(), L[flip, 1].copy()
        flip = rng.random(n) < 0.1
        L[flip, 2], H[flip, 2] = H[flip, 2].copy(), L[flip, 2].copy()
    return L, H


@pytest.mark.parametrize("kind", ["mixed", "aligned", "flat", "inverted_yz", "large"])
def test_sap_pairs_binned_edge_cases(sdlib, orc, kind):
    """The binned sweep (columns, one report per pair in the column of the
    overlap's lower y-z corner) finds exactly the oracle's pair set."""
    import torch
    L, H = _scene(kind, 20_000 if kind != "flat" else 4000, seed=len(kind))
    want = orc.aabb_pairs(L, H)
    got, cnt, err = sdlib.SweepAndPrune.pairs(torch.from_numpy(L).cuda(), torch.from_numpy(H).cuda(), len(want) + 8)
    assert err == 0 and cnt == len(want), (kind, cnt, len(want), err)
    assert np.array_equal(got.cpu().numpy().view(np.uint64), want)
