"""The rotating drum: spheres and rigid clumps against a triangle mesh that
turns about its axis, on the GPU against the CPU oracle (which tests every
triangle of the mesh, so the GPU's grid-pruned candidates must give the same
contacts), bit-exactly, including the mesh pose."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def small_drum(sd, omega=20.0, seed=0, engine=None):
    from stardust_gb300 import scenes
    d = scenes.drum_scene(n_spheres=650, radius=0.04, length=0.04, n_around=24, n_along=6, n_rings=3,
                          r_range=(0.002, 0.0028), omega=omega, seed=seed)
    if engine is not None:
        d["cfg"].collision_engine = engine
    eng = sd.DEMEngine(d["cfg"])
    scenes.add_drum_scene(eng, d)
    eng.prepare()
    eng.step(d["dt"], 0)  # builds the step (and the mesh's per-step rotation)
    eng.sync()
    return eng, d


def body_tables(d, n):
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
    return body_of, r0, np.array(first, np.uint32), np.array(count, np.uint32)


@pytest.mark.parametrize("steps", [1, 50, 400])
@pytest.mark.parametrize("engine", ["SHP", "SAP"])
def test_drum_bit_exact(sdlib, orc, steps, engine):
    """Either collision engine: sphere-triangle candidates from the mesh's
    static grid (SHP) or from sweep and prune along the drum axis (SAP)."""
    from stardust_gb300 import _abi
    eng, d = small_drum(sdlib, engine=getattr(_abi, "SD_ENGINE_" + engine))
    n = eng.n
    body_of, r0, first, count = body_tables(d, n)
    pos, vel, omg = eng.positions(), eng.velocities(), eng.omegas()
    ids = np.arange(n, dtype=np.uint32)
    omg.view(np.uint32)[:, 3] = np.where(body_of >= 0, ids | np.uint32(0x80000000), ids)
    b0 = {"pos": eng.bodies(_abi.SD_BODY_POSITION), "vel": eng.bodies(_abi.SD_BODY_VELOCITY),
          "quat": eng.bodies(_abi.SD_BODY_QUATERNION), "omega": eng.bodies(_abi.SD_BODY_OMEGA),
          "angmom": eng.bodies(_abi.SD_BODY_ANGMOM), "inv": eng.bodies(_abi.SD_BODY_INV_INERTIA),
          "first": first, "count": count}
    mesh = orc.make_mesh(d["tris"], d["patch"], d["centre"], eng.mesh_state())
    p = orc.params_checked(d["cfg"], pos[:, 3], d["dt"], eng.params())
    op, ov, ow, ob = orc.run_full(p, pos, vel, omg, steps, b0, r0, body_of, mesh)
    eng.step(d["dt"], steps)
    eng.sync()
    assert eng.stats()["device_errors"] == 0
    un = lambda a: orc.unsort(a, ow)
    assert np.array_equal(bits(eng.positions()), bits(un(op)))
    assert np.array_equal(bits(eng.velocities()), bits(un(ov)))
    assert np.array_equal(bits(eng.bodies(_abi.SD_BODY_QUATERNION)), bits(ob["quat"]))
    assert np.array_equal(bits(eng.mesh_state()), bits(np.array(mesh.state, np.float32)))
    eng.close()


def test_drum_keeps_spheres_inside_and_drags_the_bed(sdlib):
    """The bed stays inside the turning cylinder and picks up angular
    momentum about the drum axis in the drum's sense of rotation."""
    eng, d = small_drum(sdlib, omega=30.0, seed=1)
    eng.step(d["dt"], 20000)
    eng.sync()
    assert eng.stats()["device_errors"] == 0
    p = eng.positions().astype(np.float64)
    v = eng.velocities().astype(np.float64)
    c = np.array(d["centre"])
    rad = np.hypot(p[:, 1] - c[1], p[:, 2] - c[2])
    assert np.all(rad + p[:, 3] < 0.04 * 1.01)
    assert np.all(np.abs(p[:, 0] - c[0]) + p[:, 3] < 0.02 * 1.01)
    # angular momentum about the x axis through the centre: sense of +omega
    Lx = (v[:, 3] * ((p[:, 1] - c[1]) * v[:, 2] - (p[:, 2] - c[2]) * v[:, 1])).sum()
    assert Lx > 0
    eng.close()
