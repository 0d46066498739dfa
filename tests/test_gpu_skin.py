"""Skin contact lists (knob skin_um) against the oracle: the lists change
which candidates a sphere tests, never the contact set or its order, so
every state stays bit-identical -- across builds forced by motion, by
set_state, overflowing lists (dense packs), and the re-sort's fallback."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def scene(n, inflate, speed, seed):
    from stardust_gb300 import scenes
    pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=scenes.scaled_box(n), seed=seed)
    pos = pos.copy()
    vel = vel.copy()
    pos[:, 3] *= np.float32(inflate)
    cfg.cell = float(2 * pos[:, 3].max())
    rng = np.random.default_rng(seed)
    vel[:, :3] = (rng.standard_normal((n, 3)) * speed).astype(np.float32)
    return pos, vel, cfg, dt


@pytest.mark.parametrize("skin_um,inflate,speed", [(50, 1.0, 2.0), (1000, 1.0, 0.5), (200, 1.3, 5.0),
                                                   (2000, 1.8, 1.0), (20, 1.2, 20.0)])
def test_skin_lists_bit_exact(sdlib, orc, skin_um, inflate, speed):
    from stardust_gb300 import _abi
    old = _abi.tune_get("skin_um")
    try:
        _abi.tune_set("skin_um", skin_um)
        n = 20_000
        pos, vel, cfg, dt = scene(n, inflate, speed, seed=skin_um)
        eng = sdlib.DEMEngine(cfg)
        eng.add_spheres(pos, vel)
        eng.prepare()
        steps = 40
        eng.step(dt, steps)
        eng.sync()
        assert eng.stats()["device_errors"] == 0
        p = orc.params_from_engine(eng.params(), dt)
        op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(n)), steps)
        assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
        assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
        assert np.array_equal(bits(eng.omegas())[:, :3], bits(orc.unsort(ow, ow))[:, :3])
        eng.close()
    finally:
        _abi.tune_set("skin_um", old)


def test_skin_lists_after_set_state(sdlib):
    """Positions written by the host force a build: the run matches one
    without lists."""
    from stardust_gb300 import _abi
    A = _abi
    old = _abi.tune_get("skin_um")
    out = []
    try:
        for skin in (0, 500):
            _abi.tune_set("skin_um", skin)
            pos, vel, cfg, dt = scene(20_000, 1.2, 0.5, seed=9)
            eng = sdlib.DEMEngine(cfg)
            eng.add_spheres(pos, vel)
            eng.prepare()
            eng.step(dt, 10)
            x = eng.positions()
            x[:, :3] += np.float32(3e-4)  # beyond the skin: stale lists would miss contacts
            eng.set(A.SD_FIELD_POSITION, x)
            eng.step(dt, 10)
            eng.sync()
            out.append((eng.positions(), eng.velocities()))
            eng.close()
    finally:
        _abi.tune_set("skin_um", old)
    assert np.array_equal(bits(out[0][0]), bits(out[1][0]))
    assert np.array_equal(bits(out[0][1]), bits(out[1][1]))
