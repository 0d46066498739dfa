"""The index arithmetic of the incremental re-sort, restated in Python and
checked against a stable sort on random cases (no GPU).  The kernels it
mirrors: the positions of the moved entries and the slot - rank list
(sd_resort.cu, resort_scan_kernel's last block), the source slot of every
sorted position (sd_dem.cu, sorted_entry) and the cell-table shift
(sd_dem.cu, dem_fix_gather_kernel).  The GPU tests check the kernels
themselves against the oracle bit for bit; this one pins the invariants
the design rests on: unmoved slots keep their relative order, so the new
order is a merge of two sorted sequences."""
import bisect

import numpy as np
import pytest


def resort_order(keys_prev, keys_new, ncells):
    """Sorted position -> source slot, and the shifted cell table, by the
    re-sort's rules."""
    n = len(keys_prev)
    cell_start = np.searchsorted(keys_prev, np.arange(ncells + 1), side="left")
    moved = [s for s in range(n) if keys_new[s] != keys_prev[s]]
    lst = sorted((int(keys_new[s]), s) for s in moved)          # (key, slot) order
    slots = sorted(moved)
    pos = []
    for r, (key, slot) in enumerate(lst):
        lo, hi = min(cell_start[min(key, ncells)], n), min(cell_start[min(key + 1, ncells)], n)
        x = min(max(slot, lo), hi)                                # unmoved slots before: x - moved below x
        pos.append(r + x - bisect.bisect_left(slots, x))
    q = [s - j for j, s in enumerate(slots)]
    src = []
    for k in range(n):
        lo = bisect.bisect_left(pos, k)
        if lo < len(pos) and pos[lo] == k:
            src.append(lst[lo][1])
        else:
            u = k - lo                                            # unmoved rank
            src.append(u + bisect.bisect_right(q, u))
    cs = cell_start.astype(np.int64).copy()
    for s in moved:                                               # one entry from key a to key b
        a, b = int(keys_prev[s]), int(keys_new[s])
        cs[min(a, b) + 1:max(a, b) + 1] += -1 if b > a else 1
    return src, cs


@pytest.mark.parametrize("seed", range(6))
def test_resort_order_is_the_stable_sort(seed):
    rng = np.random.default_rng(seed)
    for _ in range(200):
        n = int(rng.integers(1, 200))
        ncells = int(rng.integers(1, 50))
        keys_prev = np.sort(rng.integers(0, ncells, n))
        keys_new = keys_prev.copy()
        m = int(rng.integers(0, min(n, 40) + 1))
        idx = rng.choice(n, m, replace=False)
        keys_new[idx] = rng.integers(0, ncells, m)
        src, cs = resort_order(keys_prev, keys_new, ncells)
        assert src == sorted(range(n), key=lambda i: (keys_new[i], i))
        assert np.array_equal(cs, np.searchsorted(np.sort(keys_new), np.arange(ncells + 1), side="left"))
