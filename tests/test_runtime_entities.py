"""Runtime add/remove of entities (the reference's
EntityHandler::addEntityRuntime is a stub, entity_handler.cpp:116-119).
Host-side rules run on the CPU; on the GPU, a run that continues after a
change matches the oracle started from the changed state, bit for bit, and
the step count and the mesh pose carry over."""
import numpy as np
import pytest


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_remove_before_prepare_and_argument_checks(sdlib):
    eng = sdlib.DEMEngine()
    pos = np.array([[0.1 * k, 0.5, 0.5, 0.01] for k in range(1, 6)], np.float32)
    vel = np.array([[k, 0, 0, 1e-3] for k in range(1, 6)], np.float32)
    eng.add_spheres(pos, vel)
    eng.add_clump(np.array([[0.01, 0, 0, 0.01], [-0.01, 0, 0, 0.01]], np.float32), 2e-3, (0.5, 0.2, 0.5))
    eng.add_spheres(pos[:1] + np.float32([0, 0.3, 0, 0]), vel[:1])
    assert eng.n == 8
    for bad, what in (([9], "out of range"), ([1, 1], "twice"), ([5], "clump")):
        with pytest.raises(sdlib.SdError) as e:
            eng.remove_spheres(bad)
        assert what in str(e.value)
    eng.remove_spheres([0, 3])
    assert eng.n == 6
    eng.close()




def run_oracle(orc, eng, dt, steps):
    p = orc.params_checked(eng.config, eng.positions()[:, 3], dt, eng.params())
    n = eng.n
    return orc.run(p, eng.positions(), eng.velocities(), orc.with_ids(eng.omegas(), np.arange(n)), steps)


@pytest.mark.gpu
def test_add_and_remove_spheres_at_runtime(sdlib, orc):
    from stardust_gb300 import scenes
    pos, vel, cfg, dt = scenes.box_lattice(n_side=10, seed=3)
    eng = sdlib.DEMEngine(cfg)
    eng.add_spheres(pos, vel)
    eng.prepare()
    eng.step(dt, 30)
    # add a layer of new spheres above the lattice
    rng = np.random.default_rng(0)
    k = 60
    new = np.zeros((k, 4), np.float32)
    new[:, :2] = rng.uniform(0.1, 0.5, (k, 2))
    new[:, 2] = 0.55
    new[:, 3] = 0.01
    nv = np.zeros((k, 4), np.float32)
    nv[:, 2] = -0.5
    nv[:, 3] = 1e-3
    eng.add_spheres(new, nv)
    assert eng.n == len(pos) + k and eng.stats()["steps"] == 30
    assert np.array_equal(bits(eng.positions()[len(pos):]), bits(new))
    op, ov, ow = run_oracle(orc, eng, dt, 40)
    eng.step(dt, 40)
    eng.sync()
    assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
    assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
    # remove every third sphere: the rest keep order and state
    before = eng.positions()
    gone = np.arange(0, eng.n, 3)
    eng.remove_spheres(gone)
    keep = np.setdiff1d(np.arange(len(before)), gone)
    assert eng.n == len(keep) and np.array_equal(bits(eng.positions()), bits(before[keep]))
    op, ov, ow = run_oracle(orc, eng, dt, 40)
    eng.step(dt, 40)
    eng.sync()
    assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
    assert eng.stats()["steps"] == 110 and eng.stats()["device_errors"] == 0
    eng.close()


@pytest.mark.gpu
def test_runtime_change_keeps_bodies_and_mesh_pose(sdlib, orc):
    from stardust_gb300 import _abi, scenes
    d = scenes.drum_scene(n_spheres=650, radius=0.04, length=0.04, n_around=24, n_along=6, n_rings=3,
                          r_range=(0.002, 0.0028), omega=20.0, seed=5)
    eng = sdlib.DEMEngine(d["cfg"])
    scenes.add_drum_scene(eng, d)
    eng.prepare()
    eng.step(d["dt"], 200)
    eng.sync()
    mesh_before = eng.mesh_state()
    q_before = eng.bodies(_abi.SD_BODY_QUATERNION)
    nbody_spheres = sum(len(c[0]) for c in d["clumps"])
    free = np.arange(nbody_spheres, eng.n)
    eng.remove_spheres(free[::4])
    assert np.array_equal(bits(eng.mesh_state()), bits(mesh_before))
    assert np.array_equal(bits(eng.bodies(_abi.SD_BODY_QUATERNION)), bits(q_before))
    # the continued run against the oracle from the changed state
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
    op, ov, ow, ob = orc.run_full(p, pos, vel, omg, 150, b0, r0, body_of, mesh)
    eng.step(d["dt"], 150)
    eng.sync()
    assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
    assert np.array_equal(bits(eng.bodies(_abi.SD_BODY_QUATERNION)), bits(ob["quat"]))
    assert np.array_equal(bits(eng.mesh_state()), bits(np.array(mesh.state, np.float32)))
    eng.close()
