"""The column rule of the binned exact sweep (stardust_gb300/csrc/sd_sap.cu)
restated in numpy float32 and checked on the CPU: columns at least 1.0001 x
the largest y or z extent wide span at most two columns per box and axis,
and every overlapping pair is reported in exactly one column -- the column
of its overlap's lower y-z corner, which lies in both boxes' column ranges.
The GPU operator itself is compared with the oracle's pair sets in
tests/test_gpu_sap.py."""
import numpy as np
import pytest

F = np.float32
KMAX = 255


def grid(lo, hi):
    ly, hy = np.minimum(lo[:, 1], hi[:, 1]), np.maximum(lo[:, 1], hi[:, 1])
    lz, hz = np.minimum(lo[:, 2], hi[:, 2]), np.maximum(lo[:, 2], hi[:, 2])
    y0, y1, z0, z1 = ly.min(), hy.max(), lz.min(), hz.max()
    ext = max((hy - ly).max(), (hz - lz).max())
    c = max(F(ext * F(1.0001)), F((y1 - y0) / F(KMAX)), F((z1 - z0) / F(KMAX)))
    if not (c > 0 and np.isfinite(c)):
        return F(0), F(0), F(0), 1, 1
    inv = F(F(1) / c)
    gy = min(KMAX, max(1, int(min(F((y1 - y0) * inv), F(1e6))) + 1))
    gz = min(KMAX, max(1, int(min(F((z1 - z0) * inv), F(1e6))) + 1))
    return F(y0), F(z0), inv, gy, gz


def col(v, v0, inv, g):
    t = np.floor(F(F(v - v0) * inv))
    return np.where(t >= 0, np.where(t < g, t, g - 1), 0).astype(np.int64)


def boxes(kind, n, seed):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-0.7, 1.3, (n, 3)).astype(F)
    h = np.exp(rng.normal(np.log(0.01), 0.6, (n, 3))).astype(F)
    if kind == "aligned":
        c = (rng.integers(0, 64, (n, 3)) / 32.0).astype(F)
        h = (rng.integers(0, 3, (n, 3)) / 64.0).astype(F)
    elif kind == "large":
        c = (c * F(1000) + F(1e6)).astype(F)
        h = (h * F(1000)).astype(F)
    elif kind == "big":
        h[rng.random(n) < 0.01] = F(0.7)
    lo, hi = (c - h).astype(F), (c + h).astype(F)
    if kind == "inverted":
        f = rng.random(n) < 0.2
        lo[f, 1], hi[f, 1] = hi[f, 1].copy(), lo[f, 1].copy()
    return lo, hi


@pytest.mark.parametrize("kind", ["uniform", "aligned", "large", "big", "inverted"])
def test_each_overlapping_pair_is_reported_in_one_column(kind):
    lo, hi = boxes(kind, 1500, seed=len(kind))
    y0, z0, inv, gy, gz = grid(lo, hi)
    ly, hy = np.minimum(lo[:, 1], hi[:, 1]), np.maximum(lo[:, 1], hi[:, 1])
    lz, hz = np.minimum(lo[:, 2], hi[:, 2]), np.maximum(lo[:, 2], hi[:, 2])
    cy0, cy1 = col(ly, y0, inv, gy), col(hy, y0, inv, gy)
    cz0, cz1 = col(lz, z0, inv, gz), col(hz, z0, inv, gz)
    assert (cy1 - cy0).max() <= 1 and (cz1 - cz0).max() <= 1  # at most 2 x 2 columns per box
    # overlapping pairs by the operator's closed-box test
    ov = ((lo[None, :, 1] <= hi[:, None, 1]) & (lo[:, None, 1] <= hi[None, :, 1]) &
          (lo[None, :, 2] <= hi[:, None, 2]) & (lo[:, None, 2] <= hi[None, :, 2]))
    i, j = np.nonzero(np.triu(ov, 1))
    assert len(i) > 0
    my = np.maximum(ly[i], ly[j])
    mz = np.maximum(lz[i], lz[j])
    ry, rz = col(my, y0, inv, gy), col(mz, z0, inv, gz)
    # the reporting column lies in both boxes' column ranges, so the pair is
    # swept in it (once: a pair meets in one column only once)
    for a in (i, j):
        assert np.all((cy0[a] <= ry) & (ry <= cy1[a]) & (cz0[a] <= rz) & (rz <= cz1[a]))
