"""The bench workloads at their full sizes against the CPU oracle, bit for
bit: the 1,048,576-sphere settling box (as benchmarked, and with inflated
radii so that contacts are everywhere) and the 2,097,152-sphere rotating
drum with clumps and its 20,480-triangle mesh.  The oracle's OpenMP step is
fast enough (tens of ms per step at these sizes) to check a few steps
exactly instead of only size-independent properties."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("inflate", [1.0, 1.2])
def test_settling_box_1m_bit_exact(sdlib, orc, inflate):
    from stardust_gb300 import scenes
    pos, vel, cfg, dt, phi = scenes.settling_rsa(1 << 20, box=(1.0, 1.0, 2.0), seed=0)
    pos = pos.copy()
    pos[:, 3] *= np.float32(inflate)
    cfg.cell = float(2 * pos[:, 3].max())
    cfg.pair_capacity = 1 << 23  # the dense variant holds ~2.1M contact pairs
    eng = sdlib.DEMEngine(cfg)
    eng.add_spheres(pos, vel)
    eng.prepare()
    steps = 4
    p = orc.params_checked(cfg, pos[:, 3], dt, eng.params())
    n = len(pos)
    if inflate > 1.0:  # the dense state's contact list first
        sp, sv, sw, _, cs = orc.prepare(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(n)))
        want = orc.contact_pairs(p, sp, sw, cs, cap=1 << 24)
        got = eng.pairs(cap=1 << 24)
        assert len(want) > n and np.array_equal(got, want)
    op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(n)), steps)
    eng.step(dt, steps)
    eng.sync()
    assert eng.stats()["device_errors"] == 0
    assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
    assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
    uw = orc.unsort(ow, ow)
    uw[:, 3] = 0
    assert np.array_equal(bits(eng.omegas()), bits(uw))
    eng.close()


def test_drum_2m_bit_exact(sdlib, orc):
    from stardust_gb300 import _abi, scenes
    d = scenes.drum_scene()
    eng = sdlib.DEMEngine(d["cfg"])
    scenes.add_drum_scene(eng, d)
    eng.prepare()
    eng.step(d["dt"], 0)
    eng.sync()
    n = eng.n
    body_of = np.full(n, -1, np.int32)
    r0 = np.zeros((n, 4), np.float32)
    first, count = [], []
    i = 0
    for b, (rel, *_r) in enumerate(d["clumps"]):
        first.append(i)
        count.append(len(rel))
        body_of[i:i + len(rel)] = b
        r0[i:i + len(rel), :3] = rel[:, :3]
        i += len(rel)
    pos, vel, omg = eng.positions(), eng.velocities(), eng.omegas()
    ids = np.arange(n, dtype=np.uint32)
    omg.view(np.uint32)[:, 3] = np.where(body_of >= 0, ids | np.uint32(0x80000000), ids)
    b0 = {"pos": eng.bodies(_abi.SD_BODY_POSITION), "vel": eng.bodies(_abi.SD_BODY_VELOCITY),
          "quat": eng.bodies(_abi.SD_BODY_QUATERNION), "omega": eng.bodies(_abi.SD_BODY_OMEGA),
          "angmom": eng.bodies(_abi.SD_BODY_ANGMOM), "inv": eng.bodies(_abi.SD_BODY_INV_INERTIA),
          "first": np.array(first, np.uint32), "count": np.array(count, np.uint32)}
    t, pa, c = eng.mesh()
    mesh = orc.make_mesh_frame(t, pa, eng.mesh_state())
    p = orc.params_checked(d["cfg"], pos[:, 3], d["dt"], eng.params())
    steps = 3
    op, ov, ow, ob = orc.run_full(p, pos, vel, omg, steps, b0, r0, body_of, mesh)
    eng.step(d["dt"], steps)
    eng.sync()
    assert eng.stats()["device_errors"] == 0
    assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
    assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
    assert np.array_equal(bits(eng.bodies(_abi.SD_BODY_QUATERNION)), bits(ob["quat"]))
    assert np.array_equal(bits(eng.mesh_state()), bits(np.array(mesh.state, np.float32)))
    eng.close()
