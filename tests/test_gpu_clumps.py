"""Rigid clumps on the GPU against the CPU oracle, through the C ABI.

A clump is a rigid body made of spheres (DEMParticle, entity.cpp:9-59, and
the rigid-body kernels of physics_update.cu:26-310).  Its spheres collide
like free spheres (pairs within one body skipped, collision_resolution.cu:69);
their contact forces and torques are gathered per body, the body is advanced,
and its spheres are placed from the new pose.  Every float operation is
specified, so the sphere state and the body state are compared bit-exactly
with oracle/sd_oracle.c:sdo_run_bodies."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLAG = np.uint32(0x80000000)


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def build(sd, n_side=6, seed=0, free_fraction=0.25, gravity=None, walls=None, spacing=4.6):
    """clump_box at a spacing where neighbouring clumps start in contact."""
    from stardust_gb300 import scenes
    clumps, fp, fv, cfg, dt = scenes.clump_box(n_side, free_fraction, seed, spacing)
    if gravity is not None:
        cfg.gravity = gravity
    if walls is not None:
        cfg.walls = walls
    eng = sd.DEMEngine(cfg)
    scenes.add_clump_scene(eng, clumps, fp, fv)
    eng.prepare()
    eng.sync()
    body_of = np.full(eng.n, -1, np.int32)
    r0 = np.zeros((eng.n, 4), np.float32)
    first, count = [], []
    i = 0
    for b, (rel, *_rest) in enumerate(clumps):
        first.append(i)
        count.append(len(rel))
        body_of[i:i + len(rel)] = b
        r0[i:i + len(rel), :3] = rel[:, :3]
        i += len(rel)
    return eng, dt, body_of, r0, np.array(first, np.uint32), np.array(count, np.uint32)


def body_state(sd, eng):
    from stardust_gb300 import _abi
    return {"pos": eng.bodies(_abi.SD_BODY_POSITION), "vel": eng.bodies(_abi.SD_BODY_VELOCITY),
            "quat": eng.bodies(_abi.SD_BODY_QUATERNION), "omega": eng.bodies(_abi.SD_BODY_OMEGA),
            "angmom": eng.bodies(_abi.SD_BODY_ANGMOM), "inv": eng.bodies(_abi.SD_BODY_INV_INERTIA)}


def oracle_input(orc, eng, body_of):
    """The engine's uploaded state in id order, ids (with the clump flag) in omega.w."""
    pos, vel, omg = eng.positions(), eng.velocities(), eng.omegas()
    ids = np.arange(eng.n, dtype=np.uint32)
    ids = np.where(body_of >= 0, ids | FLAG, ids)
    omg = omg.copy()
    omg.view(np.uint32)[:, 3] = ids
    return pos, vel, omg


def unsort(orc, arr, omg):
    out = np.empty_like(arr)
    out[orc.ids_of(omg)] = arr
    return out


@pytest.mark.parametrize("steps", [1, 10, 150])
def test_clumps_bit_exact(sdlib, orc, steps):
    eng, dt, body_of, r0, first, count = build(sdlib)
    assert eng.n_bodies == len(first) > 0
    pos, vel, omg = oracle_input(orc, eng, body_of)
    b0 = body_state(sdlib, eng)
    b0.update(first=first, count=count)
    p = orc.params_checked(eng.config, pos[:, 3], dt, eng.params())
    op, ov, ow, ob = orc.run_bodies(p, pos, vel, omg, steps, b0, r0, body_of)
    eng.step(dt, steps)
    eng.sync()
    assert eng.stats()["device_errors"] == 0
    uw = unsort(orc, ow, ow)
    uw[:, 3] = 0
    assert np.array_equal(bits(eng.positions()), bits(unsort(orc, op, ow)))
    assert np.array_equal(bits(eng.velocities()), bits(unsort(orc, ov, ow)))
    assert np.array_equal(bits(eng.omegas()), bits(uw))
    b1 = body_state(sdlib, eng)
    for k in ("pos", "vel", "quat", "omega", "angmom"):
        assert np.array_equal(bits(b1[k]), bits(ob[k])), k
    # the bodies moved and collided
    assert not np.array_equal(b1["quat"], b0["quat"])
    eng.close()


def test_clumps_every_knob_setting(sdlib, orc):
    """Both contact-scan variants hand clump forces to the body kernel identically."""
    from stardust_gb300 import _abi
    old = (_abi.tune_get("contact_mode"), _abi.tune_get("sort_items"))
    try:
        outs = []
        for mode, items in ((0, 8), (1, 16)):
            _abi.tune_set("contact_mode", mode)
            _abi.tune_set("sort_items", items)
            eng, dt, *_ = build(sdlib, n_side=7, seed=3)
            eng.step(dt, 40)
            eng.sync()
            outs.append((eng.positions(), eng.bodies(_abi.SD_BODY_QUATERNION)))
            eng.close()
        assert np.array_equal(bits(outs[0][0]), bits(outs[1][0]))
        assert np.array_equal(bits(outs[0][1]), bits(outs[1][1]))
    finally:
        _abi.tune_set("contact_mode", old[0])
        _abi.tune_set("sort_items", old[1])


def test_free_flight_conserves_angular_momentum(sdlib):
    """No gravity, no walls, bodies far apart: L is unchanged bit for bit,
    the quaternion stays normalised, the spheres keep their body-frame
    distances and the centre moves on a straight line."""
    from stardust_gb300 import _abi
    cfg = sdlib.EngineConfig(box_lo=(0, 0, 0), box_hi=(1, 1, 1), walls=0, cell=0.02, kn=1e5, restitution=0.5,
                             mu=0.3, gravity=(0.0, 0.0, 0.0))
    eng = sdlib.DEMEngine(cfg)
    rel = np.array([[0.02, 0, 0, 0.01], [-0.01, 0.015, 0, 0.01], [-0.01, -0.015, 0.005, 0.01]], np.float32)
    rel[:, :3] -= rel[:, :3].mean(axis=0)
    eng.add_clump(rel, 0.01, (0.5, 0.5, 0.5), (0.1, 0.0, 0.05), (3.0, -7.0, 11.0))
    eng.prepare()
    L0 = eng.bodies(_abi.SD_BODY_ANGMOM).copy()
    dt, steps = 1e-4, 2000
    eng.step(dt, steps)
    eng.sync()
    assert np.array_equal(bits(eng.bodies(_abi.SD_BODY_ANGMOM)), bits(L0))
    q = eng.bodies(_abi.SD_BODY_QUATERNION)[0].astype(np.float64)
    assert abs(np.linalg.norm(q) - 1.0) < 1e-6
    pos = eng.positions()[:, :3].astype(np.float64)
    d_now = np.linalg.norm(pos[:, None] - pos[None], axis=-1)
    d_ref = np.linalg.norm(rel[:, None, :3] - rel[None, :, :3], axis=-1)
    assert np.allclose(d_now, d_ref, atol=2e-6)
    c = eng.bodies(_abi.SD_BODY_POSITION)[0, :3].astype(np.float64)
    assert np.allclose(c, [0.5 + 0.1 * dt * steps, 0.5, 0.5 + 0.05 * dt * steps], atol=1e-4)
    eng.close()


def test_pairs_skip_same_body(sdlib, orc):
    """The contact pair list has no pair of one body's (overlapping) spheres."""
    eng, dt, body_of, *_ = build(sdlib, n_side=5, seed=7, free_fraction=0.0, gravity=(0.0, 0.0, 0.0))
    pairs = eng.pairs()
    a = (pairs >> np.uint64(32)).astype(np.int64)
    b = (pairs & np.uint64(0xFFFFFFFF)).astype(np.int64)
    assert len(pairs) == 0 or not np.any((body_of[a] >= 0) & (body_of[a] == body_of[b]))
    # the spheres of one clump do overlap, so this checks the skip
    pos = eng.positions()
    first = np.flatnonzero(body_of == 0)
    d = np.linalg.norm(pos[first[0], :3] - pos[first[1], :3])
    assert d < pos[first[0], 3] + pos[first[1], 3]
    eng.close()


def test_clump_checkpoint_resume_bit_exact(sdlib, tmp_path):
    from stardust_gb300 import _abi
    eng, dt, *_ = build(sdlib, seed=5)
    eng.step(dt, 20)
    path = tmp_path / "ck.bin"
    eng.save_checkpoint(path)
    eng.step(dt, 30)
    eng.sync()
    ref_pos, ref_q = eng.positions(), eng.bodies(_abi.SD_BODY_QUATERNION)
    cfg = eng.config
    eng.close()
    e2 = sdlib.DEMEngine(cfg)
    e2.load_checkpoint(path)
    assert e2.stats()["n_bodies"] == len(ref_q)
    e2.step(dt, 30)
    e2.sync()
    assert np.array_equal(bits(e2.positions()), bits(ref_pos))
    assert np.array_equal(bits(e2.bodies(_abi.SD_BODY_QUATERNION)), bits(ref_q))
    e2.close()


def test_cube_particle_drop(sdlib):
    """DEMEngine::add(DEMParticle(grid_resolution=3)) dropped onto the floor:
    27 spheres fall as one body, stay rigid and come to rest on the floor."""
    from stardust_gb300 import _abi
    cfg = sdlib.EngineConfig(box_lo=(0, 0, 0), box_hi=(0.5, 0.5, 0.5), walls=0x3F, cell=0.05, kn=1e5,
                             restitution=0.3, mu=0.3, gravity=(0.0, 0.0, -9.81))
    eng = sdlib.DEMEngine(cfg)
    # size 0.15, diameter 0.05: floor(3)^2 = 9 -> spacing 0.15/9
    eng.add(3, 0.15, 0.05, 0.5, (0.25, 0.25, 0.2), (0.0, 0.0, 0.0))
    assert eng.n == 27 and eng.n_bodies == 1
    eng.prepare()
    p0 = eng.positions()[:, :3].astype(np.float64)
    eng.step(2e-5, 20000)
    eng.sync()
    p1 = eng.positions()[:, :3].astype(np.float64)
    d0 = np.linalg.norm(p0[:, None] - p0[None], axis=-1)
    d1 = np.linalg.norm(p1[:, None] - p1[None], axis=-1)
    assert np.allclose(d0, d1, atol=1e-5)
    r = 0.025
    assert p1[:, 2].min() > r * 0.9 and p1[:, 2].min() < r * 1.1  # resting on the floor
    v = eng.bodies(_abi.SD_BODY_VELOCITY)[0, :3]
    assert np.linalg.norm(v) < 0.05
    assert eng.stats()["device_errors"] == 0
    eng.close()


def test_clumps_under_every_resort_setting(sdlib):
    """Clump scenes through the re-sort's both orders: radix passes only
    (resort_max 0), mostly the passes with the in-place reorder's fallback
    copy (2), and the incremental order (1024) -- the same bits, body states
    included (the slot table the body kernel reads follows every order)."""
    from stardust_gb300 import _abi
    old = _abi.tune_get("resort_max")
    outs = []
    try:
        for rm in (0, 2, 1024):
            _abi.tune_set("resort_max", rm)
            eng, dt, *_ = build(sdlib, n_side=7, seed=3)
            moved = []
            for _ in range(30):
                eng.step(dt, 2)
                moved.append(eng.stats()["moved_keys"])
            eng.sync()
            assert eng.stats()["device_errors"] == 0
            outs.append((eng.positions(), eng.velocities(), eng.bodies(_abi.SD_BODY_QUATERNION),
                         eng.bodies(_abi.SD_BODY_POSITION), moved))
            eng.close()
    finally:
        _abi.tune_set("resort_max", old)
    assert max(outs[1][4]) > 2  # the fallback ran
    for o in outs[1:]:
        for a, b in zip(outs[0][:4], o[:4]):
            assert np.array_equal(bits(a), bits(b))
