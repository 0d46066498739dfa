"""The convex-hull oracle (oracle/sd_oracle_hull.c) against independent
FP64 checks: brute-force box overlap, a numpy restatement of the reference
Morton code (testLBVH.cu:113-151), linear-programming intersection tests,
and the exact penetration depth from the FP64 hull of the Minkowski
difference; and against the reference's own Morton and GJK kernels through
golden vectors they wrote on a GPU (tests/golden/ref_morton_*.npz,
ref_gjk.npz).  CPU only."""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _scene(n=1500, seed=1, spacing=0.021):
    from oracle import oracle as orc
    from stardust_gb300 import scenes
    pts, pos, quat, vel, mass, cfg, dt = scenes.hull_box(n, seed=seed, box=(0.4, 0.4, 0.4), spacing=spacing)
    return orc.hulls_from_points(pts, pos, quat, vel, mass), pts, cfg, dt


def _world_verts(H, b):
    from oracle import oracle as orc
    R = orc.matrix_from_quat(H.quat[b].astype(np.float64))
    v = H.verts[H.vstart[b]:H.vstart[b] + H.vcount[b], :3].astype(np.float64)
    return v @ R.T + H.pos[b, :3].astype(np.float64)


def test_aabb_pairs_match_brute_force(orc):
    rng = np.random.default_rng(0)
    n = 1200
    c = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    h = rng.uniform(0.005, 0.04, (n, 3)).astype(np.float32)
    lo = np.zeros((n, 4), np.float32)
    hi = np.zeros((n, 4), np.float32)
    lo[:, :3] = c - h
    hi[:, :3] = c + h
    lo[6, :3] = hi[5, :3]  # touching closed boxes count
    hi[6, :3] = hi[5, :3] + 0.01
    ov = np.all((lo[:, None, :3] <= hi[None, :, :3]) & (lo[None, :, :3] <= hi[:, None, :3]), axis=-1)
    i, j = np.nonzero(np.triu(ov, 1))
    want = np.sort((i.astype(np.uint64) << np.uint64(32)) | j.astype(np.uint64))
    got = orc.aabb_pairs(lo, hi)
    assert np.array_equal(got, want)
    assert (5 << 32 | 6) in set(got.tolist())


def test_morton_matches_restatement(orc):
    """Centroid relative to the domain centre / (domain/1024), floored,
    clamped to [-512, 511], +512, interleaved (x in bit 0)."""
    rng = np.random.default_rng(2)
    n = 5000
    c = rng.uniform(-0.2, 1.2, (n, 3)).astype(np.float32)
    lo = np.zeros((n, 4), np.float32)
    hi = np.zeros((n, 4), np.float32)
    lo[:, :3] = c - 0.01
    hi[:, :3] = c + 0.01
    glo, ghi = np.float32([0, 0, 0]), np.float32([1, 1, 1])
    got = orc.morton_ref(lo, hi, glo, ghi)
    cen = (glo + ghi) * np.float32(0.5)
    cell = (ghi - glo) / np.float32(1024)
    p = ((lo[:, :3] + hi[:, :3]) * np.float32(0.5) - cen) / cell
    d = np.where(p >= 0, np.trunc(p), np.floor(p)).astype(np.int64)
    d = np.clip(d, -512, 511) + 512

    def spread(x):
        out = np.zeros_like(x)
        for b in range(10):
            out |= ((x >> b) & 1) << (3 * b)
        return out

    want = (spread(d[:, 0]) | (spread(d[:, 1]) << 1) | (spread(d[:, 2]) << 2)).astype(np.uint32)
    assert np.array_equal(got, want)


def test_gjk_boolean_matches_linear_programming(orc):
    """GJK's intersection verdict equals LP feasibility of a common point
    (sum l_i a_i = sum m_j b_j, l, m >= 0, sum = 1) on close pairs."""
    linprog = pytest.importorskip("scipy.optimize").linprog
    H, *_ = _scene()
    lo, hi, _ = H.aabbs()
    pairs = orc.aabb_pairs(lo, hi)
    rng = np.random.default_rng(3)
    sel = pairs[rng.permutation(len(pairs))[:150]]
    agree = 0
    hits = 0
    for pr in sel:
        a, b = int(pr >> np.uint64(32)), int(pr & np.uint64(0xFFFFFFFF))
        r = H.gjk_epa(a, b)
        A, B = _world_verts(H, a), _world_verts(H, b)
        na, nb = len(A), len(B)
        Aeq = np.zeros((5, na + nb))
        Aeq[:3, :na] = A.T
        Aeq[:3, na:] = -B.T
        Aeq[3, :na] = 1
        Aeq[4, na:] = 1
        beq = np.array([0, 0, 0, 1, 1.0])
        lp = linprog(np.zeros(na + nb), A_eq=Aeq, b_eq=beq, bounds=(0, None), method="highs")
        hit = r["status"] in (1, 2)
        hits += hit
        agree += hit == (lp.status == 0)
    assert hits > 10
    assert agree == len(sel)


def test_epa_depth_matches_fp64_minkowski_hull(orc):
    """EPA depth and normal against the closest facet of the FP64 convex
    hull of all vertex differences b - a."""
    ConvexHull = pytest.importorskip("scipy.spatial").ConvexHull
    H, *_ = _scene(spacing=0.0195)
    lo, hi, _ = H.aabbs()
    pairs = orc.aabb_pairs(lo, hi)
    worst = 0.0
    checked = 0
    for pr in pairs[:400]:
        a, b = int(pr >> np.uint64(32)), int(pr & np.uint64(0xFFFFFFFF))
        r = H.gjk_epa(a, b)
        if r["status"] != 1:
            continue
        A, B = _world_verts(H, a), _world_verts(H, b)
        D = (B[None, :, :] - A[:, None, :]).reshape(-1, 3)
        hull = ConvexHull(D)
        off = -hull.equations[:, 3]  # origin distance to each facet plane (origin inside)
        k = np.argmin(off)
        depth64 = off[k]
        scale = H.iinv[a, 3] + H.iinv[b, 3]
        worst = max(worst, abs(r["depth"] - depth64) / scale)
        # the contact normal from A to B is minus the outward facet normal
        assert np.dot(-hull.equations[k, :3], r["normal"]) > 1 - 1e-4 or abs(off[np.argsort(off)[1]] - depth64) < 1e-7
        checked += 1
    assert checked > 20
    assert worst < 2e-6, worst


def test_gjk_verdicts_are_certificates(orc):
    """Whatever the seed: a separation verdict has the origin outside the FP64
    Minkowski hull (or within 1e-6 of its size of the boundary), and an
    intersection verdict with EPA depth above the contact skin has it inside
    by that depth; the final separating direction, used as a seed, ends GJK
    in one support evaluation."""
    ConvexHull = pytest.importorskip("scipy.spatial").ConvexHull
    H, *_ = _scene(spacing=0.0195)
    lo, hi, _ = H.aabbs()
    pairs = orc.aabb_pairs(lo, hi)
    rng = np.random.default_rng(5)
    n_sep = n_hit = 0
    for pr in pairs[:250]:
        a, b = int(pr >> np.uint64(32)), int(pr & np.uint64(0xFFFFFFFF))
        A, B = _world_verts(H, a), _world_verts(H, b)
        hull = ConvexHull((B[None, :, :] - A[:, None, :]).reshape(-1, 3))
        outside = hull.equations[:, 3].max()  # > 0: origin outside
        scale = float(H.iinv[a, 3] + H.iinv[b, 3])
        for seed in [None] + [rng.normal(size=3) for _ in range(3)]:
            r = H.gjk_epa(a, b, seed)
            if r["status"] == 0:
                n_sep += 1
                assert outside > -1e-6 * scale
                assert H.gjk_epa(a, b, r["dir"])["iters"] == 1
            elif r["status"] == 1 and r["depth"] > 1e-4 * scale:
                n_hit += 1
                assert abs(-outside - r["depth"]) < 1e-6 * scale
    assert n_sep > 100 and n_hit > 20


def test_hull_step_conserves_momentum(orc):
    """No gravity, no walls: pair forces cancel bit for bit, so the summed
    force is zero and linear momentum changes only by the integrator's
    rounding."""
    H, pts, cfg, dt = _scene(n=800, spacing=0.0185)
    p = orc.hull_params((0, 0, 0), (0.4, 0.4, 0.4), 1e5, orc.damp_from(1e5, 0.5), 0.3, (0, 0, 0), 1e-5, 0)
    m = H.pos[:, 3].astype(np.float64)
    p0 = (m[:, None] * H.vel[:, :3]).sum(0)
    hits = 0
    for _ in range(20):
        out = H.step(p, record=True)
        hits += int((out["status"] == 1).sum())
        fsum = out["force"][:, :3].astype(np.float64).sum(0)
        assert np.all(np.abs(fsum) < 1e-3 * np.abs(out["force"][:, :3]).max() + 1e-12)
    p1 = (m[:, None] * H.vel[:, :3]).sum(0)
    assert hits > 0
    assert np.all(np.abs(p1 - p0) < 1e-6 * np.abs(m[:, None] * H.vel[:, :3]).sum())


@pytest.mark.parametrize("case", ["a", "b"])
def test_morton_matches_reference_kernel(orc, case):
    """The restatement against computeSpaceFillingCurveCUDA itself
    (sandbox/testLBVH.cu:113-151, run on a GPU into ref_morton_<case>.npz):
    case a with a given domain (centres outside it clamp, centres below its
    centre floor), case b with the boxes' bounds as the domain."""
    g = np.load(GOLDEN / f"ref_morton_{case}.npz")
    got = orc.morton_ref(g["lo"], g["hi"], g["glo"][:3], g["ghi"][:3])
    assert np.array_equal(got, g["codes"])


def test_gjk_verdicts_match_reference_kernel(orc):
    """GJK's verdict against STARDUST::gjkCUDA's (sandbox/testGJK.cu:237-315,
    run on a GPU into ref_gjk.npz) on 600 pairs of convex point sets placed
    apart or overlapping by construction, with gaps and overlaps down to 1 %
    of their size: the oracle's status (separated / intersecting) equals the
    reference kernel's verdict and the construction on every pair."""
    g = np.load(GOLDEN / "ref_gjk.npz")
    n = len(g["counts"])
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = g["centres"]
    pos[:, 3] = 1.0
    verts = g["verts"].copy()
    iinv = np.ones((n, 4), np.float32)
    for k in range(n):
        s, c = g["starts"][k], g["counts"][k]
        verts[s:s + c, :3] -= pos[k, :3]
        iinv[k, 3] = np.linalg.norm(verts[s:s + c, :3], axis=1).max()
    quat = np.zeros((n, 4), np.float32)
    quat[:, 0] = 1.0
    z = np.zeros((n, 4), np.float32)
    H = orc.Hulls(pos, z, quat, z, z, iinv, g["starts"].astype(np.uint32), g["counts"].astype(np.uint32), verts)
    status = np.array([H.gjk_epa(a, b)["status"] for a, b in g["pairs"]])
    assert np.array_equal(g["verdict"], g["truth"])
    assert np.array_equal(status == 1, g["verdict"])
    assert np.all((status == 0) | (status == 1))
