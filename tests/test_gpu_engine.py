"""The DEM engine on the GPU against the CPU oracle, through the C ABI.

Every float operation of the step is specified (the oracle restates it
in the same order with -ffp-contract=off, the kernels are built with
-fmad=false), so positions, velocities, spins and forces are compared
BIT-EXACTLY -- tighter than the 1e-5 relative bound asked of FP32 -- and the
FP32 error against the FP64 twin of the oracle is stated and bounded."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run_engine(sd, pos, vel, cfg, dt, steps, record=True, omega=None):
    from stardust_gb300 import _abi
    cfg.flags = _abi.SD_FLAG_RECORD if record else 0
    eng = sd.DEMEngine(cfg)
    eng.add_spheres(pos, vel, omega)
    eng.prepare()
    if steps:
        eng.step(dt, steps)
    eng.sync()
    return eng


def oracle_state(orc, eng, pos, vel, dt, steps, omega=None, z_div=None):
    p = orc.params_checked(eng.config, pos[:, 3], dt, eng.params(), z_div)
    omg = orc.with_ids(np.zeros_like(pos) if omega is None else omega, np.arange(len(pos)))
    return p, orc.run(p, pos, vel, omg, steps)


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("steps", [0, 1, 7, 60])
def test_box_lattice_bit_exact(sdlib, orc, steps):
    from stardust_gb300 import scenes
    pos, vel, cfg, dt = scenes.box_lattice(n_side=16, seed=0)
    eng = run_engine(sdlib, pos, vel, cfg, dt, steps)
    p, (op, ov, ow) = oracle_state(orc, eng, pos, vel, dt, steps)
    up, uv, uw = orc.unsort(op, ow), orc.unsort(ov, ow), orc.unsort(ow, ow)
    uw[:, 3] = 0
    assert np.array_equal(bits(eng.positions()), bits(up))
    assert np.array_equal(bits(eng.velocities()), bits(uv))
    assert np.array_equal(bits(eng.omegas()), bits(uw))
    eng.close()


@pytest.mark.parametrize("contact_mode,sort_items", [(0, 8), (1, 16), (0, 16), (1, 8)])
def test_every_knob_setting_is_bit_exact(sdlib, orc, contact_mode, sort_items):
    """The autotuner's choices change speed only: each contact-scan variant
    and sort tile size gives the same bits as the oracle."""
    from stardust_gb300 import _abi, scenes
    old = (_abi.tune_get("contact_mode"), _abi.tune_get("sort_items"))
    try:
        _abi.tune_set("contact_mode", contact_mode)
        _abi.tune_set("sort_items", sort_items)
        n = 30_000
        pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=scenes.scaled_box(n), seed=11)
        pos = pos.copy()
        pos[:, 3] *= 1.2
        cfg.cell = float(2 * pos[:, 3].max())
        eng = run_engine(sdlib, pos, vel, cfg, dt, 25)
        p, (op, ov, ow) = oracle_state(orc, eng, pos, vel, dt, 25)
        assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
        assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
        eng.close()
    finally:
        _abi.tune_set("contact_mode", old[0])
        _abi.tune_set("sort_items", old[1])


@pytest.mark.parametrize("z_div", [1, 2, 8])
def test_z_division_is_bit_exact(sdlib, orc, z_div):
    """Splitting the z axis finer than x and y changes the slot order (and
    with it the summation order the oracle follows) and the candidate
    ranges, never the contact set: every split matches the oracle bit for
    bit, pairs included."""
    from stardust_gb300 import _abi, scenes
    old = _abi.tune_get("z_div")
    try:
        _abi.tune_set("z_div", z_div)
        n = 20_000
        pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=scenes.scaled_box(n), seed=5)
        pos = pos.copy()
        pos[:, 3] *= 1.25
        cfg.cell = float(2 * pos[:, 3].max())
        eng = run_engine(sdlib, pos, vel, cfg, dt, 20)
        assert eng.params()["z_div"] == z_div
        p, (op, ov, ow) = oracle_state(orc, eng, pos, vel, dt, 20, z_div=z_div)
        assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
        assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
        assert np.array_equal(bits(eng.omegas())[:, :3], bits(orc.unsort(ow, ow))[:, :3])
        sp, sv, sw, _, cs = orc.prepare(p, eng.positions(), eng.velocities(), orc.with_ids(eng.omegas(), np.arange(n)))
        pairs = eng.pairs()
        assert len(pairs) > n and np.array_equal(pairs, orc.contact_pairs(p, sp, sw, cs))
        eng.close()
    finally:
        _abi.tune_set("z_div", old)


def test_checkpoint_keeps_its_z_division(sdlib, tmp_path):
    """A checkpoint written under one z split resumes bit-exactly under
    another knob setting: the engine takes the saved split."""
    from stardust_gb300 import _abi, scenes
    old = _abi.tune_get("z_div")
    try:
        pos, vel, cfg, dt = scenes.box_lattice(n_side=12, seed=6)
        _abi.tune_set("z_div", 4)
        a = run_engine(sdlib, pos, vel, cfg, dt, 30, record=False)
        ck = tmp_path / "ck.bin"
        a.save_checkpoint(ck)
        a.step(dt, 30)
        a.sync()
        ref = a.positions(), a.velocities()
        _abi.tune_set("z_div", 1)
        c = sdlib.DEMEngine(a.config)
        c.add_spheres(pos, vel)
        c.load_checkpoint(ck)
        assert c.params()["z_div"] == 4
        c.step(dt, 30)
        c.sync()
        assert np.array_equal(bits(ref[0]), bits(c.positions()))
        assert np.array_equal(bits(ref[1]), bits(c.velocities()))
        a.close()
        c.close()
    finally:
        _abi.tune_set("z_div", old)


def test_dense_pack_forces_torques_pairs(sdlib, orc):
    """A compressed, spinning polydisperse pack with many contacts: the forces
    and torques of the step, and the contact pair set, are bit-exact."""
    from stardust_gb300 import scenes
    n = 20_000
    box = scenes.scaled_box(n)
    pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=box, seed=2)
    rng = np.random.default_rng(0)
    pos = pos.copy()
    pos[:, 3] *= 1.25  # inflate radii: overlaps everywhere
    cfg.cell = float(2 * pos[:, 3].max())
    vel = vel.copy()
    vel[:, :3] = rng.uniform(-0.2, 0.2, (n, 3))
    omega = np.zeros((n, 4), np.float32)
    omega[:, :3] = rng.uniform(-30, 30, (n, 3))
    eng = run_engine(sdlib, pos, vel, cfg, dt, 0, omega=omega)
    p = orc.params_checked(eng.config, pos[:, 3], dt, eng.params())
    omg = orc.with_ids(omega, np.arange(n))
    sp, sv, sw, _, cs = orc.prepare(p, pos, vel, omg)
    pairs_o = orc.contact_pairs(p, sp, sw, cs)
    pairs_g = eng.pairs()
    assert len(pairs_o) > n  # a dense contact network
    assert np.array_equal(pairs_g, pairs_o)
    eng.step(dt, 1)
    eng.sync()
    pn, vn, wn, keys, f, t, contacts = orc.contact_integrate(p, sp, sv, sw, cs)
    assert contacts == 2 * len(pairs_o)
    uf, ut = orc.unsort(f, sw), orc.unsort(t, sw)
    gf, gt = eng.forces(), eng.torques()
    assert np.array_equal(bits(gf), bits(uf))
    assert np.array_equal(bits(gt), bits(ut))
    assert np.array_equal(bits(eng.positions()), bits(orc.unsort(pn, sw)))
    # FP32 vs FP64 twin of the same step: stated bound
    p64 = orc.contact_integrate(p, sp.astype(np.float64), sv.astype(np.float64), sw.astype(np.float64), cs,
                                f64=True)
    f64 = orc.unsort(p64[4], sw)
    scale = np.abs(f64[:, :3]).max()
    err = np.abs(gf[:, :3].astype(np.float64) - f64[:, :3]).max() / scale
    assert err < 1e-5, err
    eng.close()


def test_checkpoint_resume_bit_exact(sdlib, orc, tmp_path):
    from stardust_gb300 import scenes
    pos, vel, cfg, dt = scenes.box_lattice(n_side=12, seed=4)
    a = run_engine(sdlib, pos, vel, cfg, dt, 40, record=False)
    a.step(dt, 40)
    a.sync()
    ref = a.positions(), a.velocities(), a.omegas()
    b = run_engine(sdlib, pos, vel, cfg, dt, 40, record=False)
    ck = tmp_path / "ck.bin"
    b.save_checkpoint(ck)
    b.close()
    c = sdlib.DEMEngine(b.config)
    c.add_spheres(pos, vel)
    c.load_checkpoint(ck)
    assert c.stats()["steps"] == 40
    c.step(dt, 40)
    c.sync()
    for x, y in zip(ref, (c.positions(), c.velocities(), c.omegas())):
        assert np.array_equal(bits(x), bits(y))
    a.close()
    c.close()


def test_set_state_resorts_only_when_keys_change(sdlib, orc):
    """Uploading the positions just read back keeps every sphere in its cell:
    no re-sort, and the run is bit-identical to one that never uploaded.
    Moving one sphere onto another, in a distant cell, re-sorts: the new
    contact is found and the pair list equals the oracle's for the new state."""
    from stardust_gb300 import _abi, scenes
    pos, vel, cfg, dt, phi = scenes.settling_rsa(20_000, box=scenes.scaled_box(20_000), seed=8)
    a = run_engine(sdlib, pos, vel, cfg, dt, 10, record=False)
    b = run_engine(sdlib, pos, vel, cfg, dt, 10, record=False)
    a.set(_abi.SD_FIELD_POSITION, a.positions())
    a.set(_abi.SD_FIELD_VELOCITY, a.velocities())
    a.step(dt, 15)
    b.step(dt, 15)
    a.sync()
    b.sync()
    assert np.array_equal(bits(a.positions()), bits(b.positions()))
    assert np.array_equal(bits(a.velocities()), bits(b.velocities()))
    # teleport sphere 0 onto the last sphere (far away: another cell)
    p = a.positions()
    far = len(p) - 1
    assert np.linalg.norm(p[0, :3] - p[far, :3]) > 4 * cfg.cell
    p[0, :3] = p[far, :3] + np.float32(0.5) * (p[0, 3] + p[far, 3]) * np.float32([1, 0, 0])
    a.set(_abi.SD_FIELD_POSITION, p)
    got = a.pairs()
    assert (np.uint64(0) << np.uint64(32) | np.uint64(far)) in set(got.tolist())
    prm = orc.params_checked(cfg, pos[:, 3], dt, a.params())
    sp, sv, sw, _, cs = orc.prepare(prm, p, a.velocities(), orc.with_ids(a.omegas(), np.arange(len(p))))
    assert np.array_equal(got, orc.contact_pairs(prm, sp, sw, cs))
    a.close()
    b.close()


def test_pinned_host_buffers_match_pageable(sdlib):
    """Page-locked host buffers are read and written in place by the kernels;
    pageable ones are staged through device memory.  Both give the same
    bits, in both directions, for every settable field."""
    import torch
    from stardust_gb300 import _abi, scenes
    pos, vel, cfg, dt, phi = scenes.settling_rsa(30_000, box=scenes.scaled_box(30_000), seed=9)
    runs = []
    for pinned in (False, True):
        rng = np.random.default_rng(1)
        eng = run_engine(sdlib, pos, vel, cfg, dt, 5, record=False)
        new = {f: eng.get(f) for f in (_abi.SD_FIELD_POSITION, _abi.SD_FIELD_VELOCITY, _abi.SD_FIELD_OMEGA)}
        new[_abi.SD_FIELD_VELOCITY][:, :3] += rng.uniform(-1e-3, 1e-3, (len(pos), 3)).astype(np.float32)
        new[_abi.SD_FIELD_OMEGA][:, :3] = 3.0
        for f, arr in new.items():
            if pinned:
                t = torch.from_numpy(np.ascontiguousarray(arr)).pin_memory()
                _abi.check(_abi.lib().sd_engine_set_state(eng._h, f, C.c_void_p(t.data_ptr()), t.numel() * 4),
                           "set_state", eng._h)
            else:
                eng.set(f, arr)
        eng.step(dt, 5)
        eng.sync()
        out = []
        for f in (_abi.SD_FIELD_POSITION, _abi.SD_FIELD_VELOCITY, _abi.SD_FIELD_OMEGA):
            if pinned:
                t = torch.empty((len(pos), 4), dtype=torch.float32).pin_memory()
                _abi.check(_abi.lib().sd_engine_get_state(eng._h, f, C.c_void_p(t.data_ptr()), t.numel() * 4),
                           "get_state", eng._h)
                out.append(t.numpy().copy())
            else:
                out.append(eng.get(f))
        runs.append(out)
        eng.close()
    for x, y in zip(*runs):
        assert np.array_equal(bits(x), bits(y))
    assert np.all(runs[0][2][:, 3] == 0)  # the id lane never leaks out


def test_set_state_and_momentum(sdlib):
    """No walls, no gravity, no friction: total momentum is conserved to
    rounding while the spheres collide."""
    from stardust_gb300 import scenes
    n = 4000
    box = scenes.scaled_box(n)
    pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=box, seed=3)
    cfg.walls = 0
    cfg.gravity = (0.0, 0.0, 0.0)
    cfg.mu = 0.0
    eng = run_engine(sdlib, pos, vel, cfg, dt, 0, record=False)
    rng = np.random.default_rng(1)
    v = vel.copy()
    v[:, :3] = rng.uniform(-1, 1, (n, 3))
    eng.set(1, v)  # SD_FIELD_VELOCITY
    assert np.array_equal(eng.velocities(), v)
    m0 = eng.stats()["momentum"]
    eng.step(dt, 200)
    st = eng.stats()
    assert st["contacts"] > 0
    mom_scale = float(np.abs(v[:, 3:4] * v[:, :3]).sum())
    assert np.allclose(st["momentum"], m0, atol=1e-5 * mom_scale)
    eng.close()


def test_restitution_head_on(sdlib):
    """Two equal spheres, head-on, no gravity or friction: the rebound speed
    ratio is the configured restitution (linear spring-dashpot, exact for
    constant damping up to the time discretisation)."""
    r, m = 0.01, 1e-3
    pos = np.array([[0.5 - r - 2.5e-4, 0.5, 0.5, r], [0.5 + r + 2.5e-4, 0.5, 0.5, r]], np.float32)
    vel = np.array([[0.5, 0, 0, m], [-0.5, 0, 0, m]], np.float32)
    from stardust_gb300 import EngineConfig
    for e in (0.2, 0.5, 0.9):
        cfg = EngineConfig(box_hi=(1, 1, 1), walls=0, gravity=(0, 0, 0), mu=0.0, restitution=e, kn=1e5)
        eng = run_engine(sdlib, pos, vel, cfg, 1e-6, 2000, record=False)
        v = eng.velocities()
        assert v[0, 0] < 0 < v[1, 0]
        assert (v[1, 0] - v[0, 0]) / 1.0 == pytest.approx(e, rel=0.01)
        eng.close()
