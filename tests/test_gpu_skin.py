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


@pytest.mark.parametrize("skin_um,inflate,speed,blocks", [(50, 1.0, 2.0, 5), (1000, 1.0, 0.5, 5), (200, 1.3, 5.0, 5),
                                                          (2000, 1.8, 1.0, 5), (20, 1.2, 20.0, 5), (200, 1.3, 5.0, 4),
                                                          (200, 1.3, 5.0, 6), (200, 1.3, 5.0, 8)])
def test_skin_lists_bit_exact(sdlib, orc, skin_um, inflate, speed, blocks):
    """Contact lists against the oracle, over skins, speeds and the list
    kernel's register budgets (knob listed_blocks)."""
    from stardust_gb300 import _abi
    old = _abi.tune_get("skin_um")
    old_blocks = _abi.tune_get("listed_blocks")
    try:
        _abi.tune_set("skin_um", skin_um)
        _abi.tune_set("listed_blocks", blocks)
        n = 20_000
        pos, vel, cfg, dt = scene(n, inflate, speed, seed=skin_um)
        eng = sdlib.DEMEngine(cfg)
        eng.add_spheres(pos, vel)
        eng.prepare()
        steps = 40
        eng.step(dt, steps)
        eng.sync()
        st = eng.stats()
        assert st["device_errors"] == 0
        # every step ran the list path (not a silent fall-back to the scan);
        # the fast scenes rebuild at every step, the slow ones use the lists
        assert st["list_builds"] >= 1 and st["list_builds"] + st["listed_steps"] == steps
        if speed * dt * 4 < 0.45e-6 * skin_um:
            assert st["listed_steps"] >= 1
        p = orc.params_checked(cfg, pos[:, 3], dt, eng.params())
        op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(n)), steps)
        assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
        assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
        assert np.array_equal(bits(eng.omegas())[:, :3], bits(orc.unsort(ow, ow))[:, :3])
        eng.close()
    finally:
        _abi.tune_set("skin_um", old)
        _abi.tune_set("listed_blocks", old_blocks)


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


def test_skin_lists_across_knob_changes(sdlib, orc):
    """Steps without the lists in between (the re-sort turned off, so the
    step graph is built without them; a lone contact stage) move spheres
    without checking their skin: the next list step must build the lists
    again.  The whole run matches the oracle bit for bit."""
    from stardust_gb300 import _abi
    old = (_abi.tune_get("skin_um"), _abi.tune_get("resort_max"))
    try:
        _abi.tune_set("skin_um", 100)
        n = 20_000
        pos, vel, cfg, dt = scene(n, 1.2, 3.0, seed=5)
        eng = sdlib.DEMEngine(cfg)
        eng.add_spheres(pos, vel)
        eng.prepare()
        eng.step(dt, 5)
        b0 = eng.stats()["list_builds"]
        _abi.tune_set("resort_max", 0)  # no re-sort: a step graph without the lists
        eng.step(dt, 15)
        _abi.tune_set("resort_max", 1024)
        eng.step(dt, 5)
        st = eng.stats()
        assert st["list_builds"] > b0  # the first list step after the change built them
        steps = 25
        eng.sync()
        assert st["device_errors"] == 0
        p = orc.params_checked(cfg, pos[:, 3], dt, eng.params())
        op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(n)), steps)
        assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
        assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
        eng.close()
    finally:
        _abi.tune_set("skin_um", old[0])
        _abi.tune_set("resort_max", old[1])


def test_coincident_spheres_are_listed(sdlib, orc):
    """Two spheres at one centre carry no contact while they coincide (no
    normal); once they separate while still overlapping, the contact acts
    -- so the lists must hold coincident partners (skipping the sphere
    itself by slot, not by distance)."""
    from stardust_gb300 import _abi, EngineConfig
    old = _abi.tune_get("skin_um")
    try:
        _abi.tune_set("skin_um", 500)
        pos = np.array([[0.5, 0.5, 0.5, 0.01], [0.5, 0.5, 0.5, 0.01], [0.3, 0.3, 0.3, 0.01]], np.float32)
        vel = np.array([[0.0, 0.0, 0.0, 1e-3], [0.2, 0.0, 0.0, 1e-3], [0.0, 0.0, 0.0, 1e-3]], np.float32)
        cfg = EngineConfig(box_lo=(0.0, 0.0, 0.0), box_hi=(1.0, 1.0, 1.0), cell=0.02, gravity=(0.0, 0.0, 0.0))
        eng = sdlib.DEMEngine(cfg)
        eng.add_spheres(pos, vel)
        eng.prepare()
        steps, dt = 30, 1e-5
        eng.step(dt, steps)
        eng.sync()
        st = eng.stats()
        # step 1 builds the lists (the pair coincides); step 2 uses them
        # (sphere 1 moved 2 um of the 225 um that force a build)
        assert st["list_builds"] >= 1 and st["listed_steps"] >= 1
        p = orc.params_checked(cfg, pos[:, 3], dt, eng.params())
        op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(3)), steps)
        v = orc.unsort(ov, ow)
        assert v[0, 0] < 0.0  # the separating pair pushed sphere 0 back
        assert np.array_equal(bits(eng.velocities()), bits(v))
        assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
        eng.close()
    finally:
        _abi.tune_set("skin_um", old)
