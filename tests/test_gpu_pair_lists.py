"""The two-kernel contact stage against the oracle.  For scenes without
clumps or meshes a pair kernel tests each candidate pair once and lists the
contacts of every sphere (up to 16); the contact kernel then applies them in
ascending slot order, which is the order of the full candidate scan, and
falls back to the scan for a sphere whose list overflowed.  Both settings of
the knob, sparse and dense packs (some spheres with more than 16 contacts),
a batch of scenes, and force recording are compared bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def packed(n, inflate, seed):
    from stardust_gb300 import scenes
    pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=scenes.scaled_box(n), seed=seed)
    pos = pos.copy()
    pos[:, 3] *= np.float32(inflate)
    cfg.cell = float(2 * pos[:, 3].max())
    cfg.pair_capacity = 1 << 22
    return pos, vel, cfg, dt


@pytest.mark.parametrize("pair_lists", [0, 1])
@pytest.mark.parametrize("inflate", [1.0, 1.3, 1.9])
def test_pair_lists_bit_exact(sdlib, orc, pair_lists, inflate):
    from stardust_gb300 import _abi
    old = (_abi.tune_get("pair_lists"), _abi.tune_get("skin_um"))
    try:
        _abi.tune_set("skin_um", 0)  # single scenes take the skin lists first
        _abi.tune_set("pair_lists", pair_lists)
        n = 20_000
        pos, vel, cfg, dt = packed(n, inflate, seed=21)
        cfg.flags = _abi.SD_FLAG_RECORD
        eng = sdlib.DEMEngine(cfg)
        eng.add_spheres(pos, vel)
        eng.prepare()
        pairs = eng.pairs()
        degree = np.bincount(np.concatenate([pairs >> 32, pairs & 0xFFFFFFFF]).astype(np.int64), minlength=n)
        if inflate > 1.5:
            assert degree.max() > 16  # some lists overflow: those spheres take the full scan
        steps = 6
        eng.step(dt, steps)
        eng.sync()
        assert eng.stats()["device_errors"] == 0
        p = orc.params_checked(cfg, pos[:, 3], dt, eng.params())
        op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(n)), steps)
        assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
        assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
        assert np.array_equal(bits(eng.omegas())[:, :3], bits(orc.unsort(ow, ow))[:, :3])
        eng.close()
    finally:
        _abi.tune_set("pair_lists", old[0])
        _abi.tune_set("skin_um", old[1])


def test_pair_lists_forces_match_single_kernel(sdlib):
    """Recorded forces and torques of a dense pack: the two-kernel stage
    gives the same bits as the single scan kernel."""
    from stardust_gb300 import _abi
    old = (_abi.tune_get("pair_lists"), _abi.tune_get("skin_um"))
    out = {}
    try:
        _abi.tune_set("skin_um", 0)
        for pl in (0, 1):
            _abi.tune_set("pair_lists", pl)
            pos, vel, cfg, dt = packed(20_000, 1.4, seed=5)
            cfg.flags = _abi.SD_FLAG_RECORD
            eng = sdlib.DEMEngine(cfg)
            eng.add_spheres(pos, vel)
            eng.prepare()
            eng.step(dt, 3)
            eng.sync()
            out[pl] = (eng.forces(), eng.torques(), eng.positions(), eng.stats()["contacts"])
            eng.close()
    finally:
        _abi.tune_set("pair_lists", old[0])
        _abi.tune_set("skin_um", old[1])
    for a, b in zip(out[0][:3], out[1][:3]):
        assert np.array_equal(bits(a), bits(b))
    assert out[0][3] == out[1][3] > 0
