"""The incremental re-sort against the oracle: the step merges the few
spheres whose cell key changed into the previous slot order instead of
radix-sorting every key, and must give exactly the stable sort's order
(the oracle's), so positions, velocities, spins and the contact list stay
bit-identical.  Scenes are set moving so that the number of changed keys
per step ranges from 0 to about a third of all spheres, on both sides of
the knob's limit (the radix passes take over above it)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def moving_scene(n, moved_per_step, seed):
    """Settling-box spheres with random velocities sized so that about
    `moved_per_step` keys change per step (a key changes when a centre
    crosses a cell face; z faces are twice as dense)."""
    from stardust_gb300 import scenes
    pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=scenes.scaled_box(n), seed=seed)
    pos = pos.copy()
    vel = vel.copy()
    rng = np.random.default_rng(seed)
    speed = moved_per_step / n * cfg.cell / (2.0 * dt)
    vel[:, :3] = (rng.standard_normal((n, 3)) * speed).astype(np.float32)
    return pos, vel, cfg, dt


@pytest.mark.parametrize("resort_max,moved", [(0, 200), (2, 200), (256, 200), (1024, 200), (1024, 0),
                                              (1024, 700), (512, 9000)])
def test_incremental_resort_bit_exact(sdlib, orc, resort_max, moved):
    from stardust_gb300 import _abi
    old = _abi.tune_get("resort_max")
    try:
        _abi.tune_set("resort_max", resort_max)
        n = 30_000
        pos, vel, cfg, dt = moving_scene(n, moved, seed=7)
        eng = sdlib.DEMEngine(cfg)
        eng.add_spheres(pos, vel)
        eng.prepare()
        steps = 12
        seen = []
        for _ in range(steps):
            eng.step(dt, 1)
            seen.append(eng.stats()["moved_keys"])
        eng.sync()
        assert eng.stats()["device_errors"] == 0
        if resort_max == 0:
            assert max(seen) == 0
        elif moved == 0:
            assert max(seen) <= 8
        else:
            assert 0.3 * moved < np.median(seen) < 3 * moved
        p = orc.params_checked(cfg, pos[:, 3], dt, eng.params())
        op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(n)), steps)
        assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
        assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
        assert np.array_equal(bits(eng.omegas())[:, :3], bits(orc.unsort(ow, ow))[:, :3])
        sp, sv, sw, _, cs = orc.prepare(p, eng.positions(), eng.velocities(),
                                        orc.with_ids(eng.omegas(), np.arange(n)))
        assert np.array_equal(eng.pairs(), orc.contact_pairs(p, sp, sw, cs))
        eng.close()
    finally:
        _abi.tune_set("resort_max", old)


def test_resort_mixes_with_radix_steps(sdlib, orc):
    """A strong gravity accelerates the spheres from rest, so the changed-key
    count grows from tens to about a thousand per step: the early steps
    re-sort incrementally, the later ones run the radix passes, and the
    state stays exact throughout."""
    from stardust_gb300 import _abi, scenes
    old = _abi.tune_get("resort_max")
    try:
        _abi.tune_set("resort_max", 256)
        n = 30_000
        pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=scenes.scaled_box(n), seed=3)
        cfg.gravity = (0.0, 0.0, -3e5)
        eng = sdlib.DEMEngine(cfg)
        eng.add_spheres(pos, vel)
        eng.prepare()
        seen = []
        for _ in range(30):
            eng.step(dt, 1)
            seen.append(eng.stats()["moved_keys"])
        assert min(seen) <= 256 < max(seen)
        p = orc.params_checked(cfg, pos[:, 3], dt, eng.params())
        op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(n)), 30)
        assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
        assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
        eng.close()
    finally:
        _abi.tune_set("resort_max", old)


def test_step_kernel_count(sdlib):
    """The plain radix step launches the contact stage, two passes and the
    reorder; with the re-sort the step adds the plan kernel (which orders the
    moved slots the contact stage listed) and the radix fallback's histogram
    (both return at once when not needed, like the passes), and the reorder
    becomes two in-place phases (gather the positions whose source moved,
    copy them back); stats report the graph's kernel nodes."""
    from stardust_gb300 import _abi
    old = _abi.tune_get("resort_max")
    counts = {}
    try:
        for rm in (0, 1024):
            _abi.tune_set("resort_max", rm)
            pos, vel, cfg, dt = moving_scene(20_000, 50, seed=1)
            eng = sdlib.DEMEngine(cfg)
            eng.add_spheres(pos, vel)
            eng.prepare()
            assert eng.stats()["step_kernels"] == 0
            eng.step(dt, 2)
            counts[rm] = eng.stats()["step_kernels"]
            eng.close()
    finally:
        _abi.tune_set("resort_max", old)
    assert counts[0] >= 4 and counts[1024] == counts[0] + 3
