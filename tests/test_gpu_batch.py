"""Batched scenes: many independent sphere boxes stepped in one launch per
stage.  Each scene's result must equal the same scene stepped alone -- the
oracle runs every scene by itself, and the batch is compared bit-exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def oracle_scene_params(orc, lo, hi, cell, cfg, dt):
    import math
    p = orc.Params()
    dims = []
    for a in range(3):
        p.lo[a], p.hi[a], p.g[a] = lo[a], hi[a], cfg.gravity[a]
        nd = math.ceil((float(np.float32(hi[a])) - float(np.float32(lo[a]))) / float(np.float32(cell)) * (1 - 1e-6))
        dims.append(max(int(nd), 1))
    p.cell = cell
    p.nx, p.ny, p.nz = dims
    p.kn, p.damp, p.mu, p.dt, p.walls = cfg.kn, orc.damp_from(cfg.kn, cfg.restitution), cfg.mu, dt, cfg.walls
    return p


@pytest.mark.parametrize("steps", [1, 30])
@pytest.mark.parametrize("skin_um,pair_lists", [(50, 2), (0, 2), (0, 0)])
def test_batch_matches_scenes_run_alone(sdlib, orc, steps, skin_um, pair_lists):
    """Three contact stages: contact lists with a skin, the pair kernel's
    lists, the plain scan."""
    from stardust_gb300 import _abi, scenes
    old = (_abi.tune_get("skin_um"), _abi.tune_get("pair_lists"))
    batch, cfg, dt = scenes.batch_boxes(n_scenes=14, seed=4, n_min=5, n_max=3000, median=400)
    try:
        _abi.tune_set("skin_um", skin_um)
        _abi.tune_set("pair_lists", pair_lists)
        eng = sdlib.DEMEngine(cfg)
        for pos, vel, lo, hi in batch:
            eng.add_scene(pos, vel, lo, hi)
        eng.prepare()
        eng.step(dt, steps)
        eng.sync()
    finally:
        _abi.tune_set("skin_um", old[0])
        _abi.tune_set("pair_lists", old[1])
    st = eng.stats()
    assert st["device_errors"] == 0
    assert st["list_builds"] + st["listed_steps"] == (steps if skin_um else 0)
    P, V = eng.positions(), eng.velocities()
    first = 0
    for pos, vel, lo, hi in batch:
        n = len(pos)
        cell = float(np.float32(2 * pos[:, 3].max()))
        p = oracle_scene_params(orc, lo, hi, cell, cfg, dt)
        op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(n)), steps)
        assert np.array_equal(bits(P[first:first + n]), bits(orc.unsort(op, ow)))
        assert np.array_equal(bits(V[first:first + n]), bits(orc.unsort(ov, ow)))
        first += n
    eng.close()


def test_batch_pairs_stay_in_their_scene(sdlib):
    from stardust_gb300 import scenes
    batch, cfg, dt = scenes.batch_boxes(n_scenes=6, seed=1, n_min=200, n_max=2000, median=800, fraction=0.45)
    eng = sdlib.DEMEngine(cfg)
    for pos, vel, lo, hi in batch:
        eng.add_scene(pos, vel, lo, hi)
    eng.prepare()
    eng.step(dt, 200)
    pairs = eng.pairs()
    edges = np.cumsum([0] + [len(b[0]) for b in batch])
    a = (pairs >> np.uint64(32)).astype(np.int64)
    b = (pairs & np.uint64(0xFFFFFFFF)).astype(np.int64)
    assert len(pairs) > 0
    assert np.array_equal(np.searchsorted(edges, a, side="right"), np.searchsorted(edges, b, side="right"))
    eng.close()
