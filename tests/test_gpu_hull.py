"""Convex hulls on the GPU against the CPU oracle, through the C ABI.

LBVH (sandbox/testLBVH.cu) pair sets and Morton codes are compared
bit-exactly with oracle/sd_oracle_hull.c; the hull step (AABBs, LBVH,
GJK/EPA per candidate entry, segmented force sum, quaternion integration)
is compared bit-exactly, state and per-entry GJK results, over several
steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _boxes(n, seed, lo=0.0, hi=1.0, hmin=0.002, hmax=0.02):
    rng = np.random.default_rng(seed)
    c = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    h = rng.uniform(hmin, hmax, (n, 3)).astype(np.float32)
    L = np.zeros((n, 4), np.float32)
    H = np.zeros((n, 4), np.float32)
    L[:, :3] = c - h
    H[:, :3] = c + h
    return L, H


@pytest.mark.parametrize("n,seed", [(0, 0), (1, 0), (2, 1), (777, 2), (50_000, 3)])
def test_lbvh_pairs_bit_exact(sdlib, orc, n, seed):
    import torch
    L, H = _boxes(n, seed, -0.3, 1.7)
    if n >= 2:
        L[1], H[1] = L[0], H[0]  # duplicate box (equal Morton codes)
    want = orc.aabb_pairs(L, H)
    cap = len(want) + 16
    got, cnt, err = sdlib.BoundingVolumes.pairs(torch.from_numpy(L).cuda(), torch.from_numpy(H).cuda(), cap)
    torch.cuda.synchronize()
    assert err == 0 and cnt == len(want)
    assert np.array_equal(got.cpu().numpy().view(np.uint64), want)


def test_lbvh_pairs_overflow_is_reported(sdlib, orc):
    import torch
    L, H = _boxes(3000, 4, hmin=0.02, hmax=0.05)
    want = orc.aabb_pairs(L, H)
    got, cnt, err = sdlib.BoundingVolumes.pairs(torch.from_numpy(L).cuda(), torch.from_numpy(H).cuda(), 10)
    assert err & sdlib._abi.SD_DEVERR_PAIR_OVERFLOW
    assert len(want) > 10


def test_lbvh_morton_bit_exact(sdlib, orc):
    import torch
    L, H = _boxes(20_000, 5, -0.5, 2.0)
    glo = L[:, :3].min(0)
    ghi = H[:, :3].max(0)
    want = orc.morton_ref(L, H, glo, ghi)
    got = sdlib.BoundingVolumes.morton(torch.from_numpy(L).cuda(), torch.from_numpy(H).cuda())
    assert np.array_equal(got.cpu().numpy().view(np.uint32), want)


def hull_engine(sd, n=3000, seed=1, spacing=0.0195, seed_mode=0, gravity=(0.0, 0.0, -9.81)):
    from stardust_gb300 import _abi, scenes
    pts, pos, quat, vel, mass, cfg, dt = scenes.hull_box(n, seed=seed, box=(0.4, 0.4, 0.4), spacing=spacing,
                                                          vmax=0.3)
    cfg.gravity = gravity
    cfg.flags = _abi.SD_FLAG_RECORD
    eng = sd.DEMEngine(cfg)
    sd.add_hull_scene(eng, pts, pos, quat, vel, mass)
    eng.prepare()
    eng.set_gjk_seed(seed_mode)
    return eng, cfg, dt


def oracle_hulls(orc, eng):
    from stardust_gb300 import _abi
    vs, vc, verts = eng.hull_shapes()
    b = {k: eng.bodies(f) for k, f in (("pos", _abi.SD_BODY_POSITION), ("vel", _abi.SD_BODY_VELOCITY),
                                         ("quat", _abi.SD_BODY_QUATERNION), ("omg", _abi.SD_BODY_OMEGA),
                                         ("ang", _abi.SD_BODY_ANGMOM), ("iinv", _abi.SD_BODY_HULL_INV_INERTIA))}
    return orc.Hulls(b["pos"], b["vel"], b["quat"], b["omg"], b["ang"], b["iinv"], vs, vc, verts)


def oracle_params(orc, cfg, dt):
    return orc.hull_params(cfg.box_lo, cfg.box_hi, cfg.kn, orc.damp_from(cfg.kn, cfg.restitution), cfg.mu,
                           cfg.gravity, dt, cfg.walls)


@pytest.mark.parametrize("steps,hull_blocks,rebuild", [(1, 4, 16), (5, 4, 16), (40, 4, 16), (40, 3, 16), (40, 4, 1),
                                                       (40, 4, 4096)])
def test_hull_steps_bit_exact(sdlib, orc, steps, hull_blocks, rebuild):
    """The hull step against the oracle; the LBVH built every step, every
    16 steps (refitted between) or once: the same pair sets and bits."""
    from stardust_gb300 import _abi
    eng, cfg, dt = hull_engine(sdlib)
    H = oracle_hulls(orc, eng)
    p = oracle_params(orc, cfg, dt)
    for _ in range(steps):
        out = H.step(p, record=True)
    old = (_abi.tune_get("hull_blocks"), _abi.tune_get("lbvh_rebuild"))
    try:
        _abi.tune_set("hull_blocks", hull_blocks)
        _abi.tune_set("lbvh_rebuild", rebuild)
        eng.step(dt, steps)
        eng.sync()
    finally:
        _abi.tune_set("hull_blocks", old[0])
        _abi.tune_set("lbvh_rebuild", old[1])
    st = eng.stats()
    assert st["device_errors"] == 0
    for k, f in (("pos", _abi.SD_BODY_POSITION), ("vel", _abi.SD_BODY_VELOCITY), ("quat", _abi.SD_BODY_QUATERNION),
                 ("omg", _abi.SD_BODY_OMEGA), ("ang", _abi.SD_BODY_ANGMOM)):
        assert np.array_equal(bits(eng.bodies(f)), bits(getattr(H, k))), k
    assert np.array_equal(bits(eng.bodies(_abi.SD_BODY_FORCE)), bits(out["force"]))
    assert np.array_equal(bits(eng.bodies(_abi.SD_BODY_TORQUE)), bits(out["torque"]))
    e = eng.hull_entries()
    assert np.array_equal(e["off"], out["off"]) and np.array_equal(e["partners"], out["partners"])
    assert np.array_equal(e["status"], out["status"]) and np.array_equal(e["iters"], out["iters"])
    hits = int((out["status"] == 1).sum())
    assert hits > 20
    uniq = e["partners"] > np.repeat(np.arange(len(e["off"]) - 1), np.diff(e["off"]))
    assert st["gjk_pairs"] == int(uniq.sum())
    assert st["gjk_iters"] == int(e["iters"][uniq].sum())
    eng.close()


def test_previous_direction_seed_cuts_iterations(sdlib, orc):
    """Seeding GJK with the pair's previous separating direction: the same
    contacts and bit-identical state (the seed only moves the iteration
    count), fewer support evaluations, and the oracle fed the same seeds
    agrees bit for bit."""
    from stardust_gb300 import _abi
    runs = {}
    for mode in (_abi.SD_GJK_SEED_PLAIN, _abi.SD_GJK_SEED_PREVIOUS):
        eng, cfg, dt = hull_engine(sdlib, seed_mode=mode)
        eng.step(dt, 30)
        H = oracle_hulls(orc, eng)
        eng.step(dt, 1)
        eng.sync()
        e = eng.hull_entries()
        st = eng.stats()
        out = H.step(oracle_params(orc, cfg, dt), off=e["off"], partners=e["partners"],
                     seeds=e["seeds"] if mode else None, record=True)
        assert np.array_equal(e["iters"], out["iters"]) and np.array_equal(e["status"], out["status"])
        assert np.array_equal(bits(eng.bodies(_abi.SD_BODY_POSITION)), bits(H.pos))
        runs[mode] = (st, e, eng.bodies(_abi.SD_BODY_POSITION))
        eng.close()
    plain, prev = runs[0], runs[2]
    # only separation certificates come from seeded runs, so the contact
    # sets, forces and states are identical
    assert np.array_equal(plain[1]["status"] == 1, prev[1]["status"] == 1)
    assert np.array_equal(bits(plain[2]), bits(prev[2]))
    mean_plain = plain[0]["gjk_iters"] / plain[0]["gjk_pairs"]
    mean_prev = prev[0]["gjk_iters"] / prev[0]["gjk_pairs"]
    assert mean_prev < 0.6 * mean_plain, (mean_plain, mean_prev)


@pytest.mark.parametrize("seed_mode", [0, 2])
def test_narrow_stage_alone_changes_nothing(sdlib, seed_mode):
    """The contact stage of a hull scene (the narrow phase of the last
    step's lists at the current bodies, launched alone for timing) changes
    no body: interleaving it leaves the bodies bit-identical, and with plain
    GJK the next steps' entries too (with seeds it moves the next step's
    seeds, so only iteration counts may differ)."""
    from stardust_gb300 import _abi
    runs = []
    for extra in (0, 3):
        eng, cfg, dt = hull_engine(sdlib, seed_mode=seed_mode)
        eng.step(dt, 5)
        for _ in range(extra):
            _abi.call("sd_engine_launch_stage", eng._h, _abi.SD_STAGE_CONTACT, 0.0, h=eng._h)
        e = eng.hull_entries()
        eng.step(dt, 5)
        eng.sync()
        assert eng.stats()["device_errors"] == 0
        runs.append((e, eng.hull_entries(), eng.bodies(_abi.SD_BODY_POSITION), eng.bodies(_abi.SD_BODY_OMEGA)))
        with pytest.raises(Exception):
            _abi.call("sd_engine_launch_stage", eng._h, _abi.SD_STAGE_SORT, 0.0, h=eng._h)
        eng.close()
    (e0, f0, p0, w0), (e1, f1, p1, w1) = runs
    assert np.array_equal(e0["off"], e1["off"]) and np.array_equal(e0["partners"], e1["partners"])
    assert np.array_equal(f0["status"] == 1, f1["status"] == 1)
    if seed_mode == 0:
        for k in ("status", "iters", "epa_iters"):
            assert np.array_equal(f0[k], f1[k]), k
        assert np.array_equal(bits(f0["dir"]), bits(f1["dir"]))
    assert np.array_equal(bits(p0), bits(p1)) and np.array_equal(bits(w0), bits(w1))


def test_lbvh_morton_matches_reference_kernel(sdlib):
    """The LBVH's Morton codes against computeSpaceFillingCurveCUDA itself
    (sandbox/testLBVH.cu:113-151, golden ref_morton_b.npz: the domain is the
    boxes' bounds, as the LBVH builds it)."""
    import torch
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "ref_morton_b.npz")
    got = sdlib.BoundingVolumes.morton(torch.from_numpy(g["lo"]).cuda(), torch.from_numpy(g["hi"]).cuda())
    assert np.array_equal(got.cpu().numpy().view(np.uint32), g["codes"])


def test_hull_gjk_verdicts_match_reference_kernel(sdlib):
    """The engine's narrow phase against STARDUST::gjkCUDA's verdicts
    (sandbox/testGJK.cu:237-315, golden ref_gjk.npz): 600 constructed pairs
    of convex point sets, apart or overlapping by 1-30 % of their size, added
    as hulls; after one step each pair is in contact (status 1) exactly when
    the reference kernel reported a collision."""
    from pathlib import Path
    from stardust_gb300 import EngineConfig
    g = np.load(Path(__file__).resolve().parent / "golden" / "ref_gjk.npz")
    cfg = EngineConfig(box_lo=(-20.0, -20.0, -20.0), box_hi=(20.0, 20.0, 20.0), walls=0, cell=4.0, kn=1e5,
                       restitution=0.5, mu=0.3, gravity=(0.0, 0.0, 0.0), pair_capacity=1 << 16)
    eng = sdlib.DEMEngine(cfg)
    for k in range(len(g["counts"])):
        s, c = int(g["starts"][k]), int(g["counts"][k])
        centre = g["centres"][k]
        eng.add_hull(g["verts"][s:s + c, :3] - centre, 1.0, tuple(float(x) for x in centre))
    eng.prepare()
    eng.step(1e-6, 1)
    eng.sync()
    assert eng.stats()["device_errors"] == 0
    e = eng.hull_entries()
    contact = set()
    for a in range(len(e["off"]) - 1):
        for q in range(e["off"][a], e["off"][a + 1]):
            if e["status"][q] == 1:
                contact.add((a, int(e["partners"][q])))
    got = np.array([(int(a), int(b)) in contact for a, b in g["pairs"]])
    assert np.array_equal(got, g["verdict"])
    eng.close()
