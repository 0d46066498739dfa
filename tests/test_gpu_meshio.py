"""Mesh entities from STL files on the GPU: the drum loaded from a binary STL
steps bit-identically to the drum built directly, and a static hopper made of
two STL meshes (placed by position and quaternion, combined into one) matches
the CPU oracle bit for bit while spheres pour through it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_drum_from_stl_is_the_drum(sdlib, tmp_path):
    from stardust_gb300 import _abi, scenes
    runs = []
    for stl in (None, tmp_path / "drum.stl"):
        d = scenes.drum_scene(n_spheres=650, radius=0.04, length=0.04, n_around=24, n_along=6, n_rings=3,
                              r_range=(0.002, 0.0028), omega=20.0, seed=2)
        eng = sdlib.DEMEngine(d["cfg"])
        scenes.add_drum_scene(eng, d, stl_path=stl)
        eng.prepare()
        eng.step(d["dt"], 300)
        eng.sync()
        assert eng.stats()["device_errors"] == 0
        runs.append((eng.positions(), eng.velocities(), eng.bodies(_abi.SD_BODY_QUATERNION), eng.mesh_state(),
                     eng.mesh()))
        eng.close()
    (a, b) = runs
    for x, y in zip(a[:4], b[:4]):
        assert np.array_equal(bits(x), bits(y))
    assert np.array_equal(bits(a[4][0]), bits(b[4][0])) and np.array_equal(a[4][1], b[4][1])


def hopper_engine(sd, tmp_path, n_side=9, engine=None):
    from stardust_gb300 import scenes
    funnel, tray = scenes.hopper_meshes()
    sd.write_stl(tmp_path / "funnel.stl", funnel, binary=False)
    # the tray is stored off-origin and rotated a quarter turn about z: its
    # placement puts it back, square, below the funnel
    q = (np.cos(np.pi / 4), 0.0, 0.0, np.sin(np.pi / 4))
    Rinv = np.array([[0.0, 1.0, 0.0], [-1.0, 0.0, 0.0], [0.0, 0.0, 1.0]], np.float32)  # rotation by -90 deg
    sd.write_stl(tmp_path / "tray.stl", (tray - np.float32([0.5, 0.5, 0.0])) @ Rinv.T)
    r = 0.004
    sp = 2.4 * r
    g = (np.arange(n_side) - (n_side - 1) / 2) * sp
    x, y, z = np.meshgrid(g, g, 0.125 + np.arange(4) * sp, indexing="ij")  # inside the funnel's mouth
    rng = np.random.default_rng(4)
    pos = np.stack([x.ravel(), y.ravel(), z.ravel(), np.full(x.size, r)], 1).astype(np.float32)
    pos[:, :3] += rng.uniform(-0.05 * r, 0.05 * r, (len(pos), 3)).astype(np.float32)
    vel = np.zeros_like(pos)
    vel[:, 3] = 2500 * 4 / 3 * np.pi * r ** 3
    cfg = sd.EngineConfig(box_lo=(-0.1, -0.1, -0.02), box_hi=(0.1, 0.1, 0.2), walls=0x3F, cell=2 * r, kn=1e4,
                          restitution=0.4, mu=0.3, gravity=(0.0, 0.0, -9.81))
    if engine is not None:
        cfg.collision_engine = engine
    eng = sd.DEMEngine(cfg)
    eng.add_spheres(pos, vel)
    eng.add_mesh_stl(tmp_path / "funnel.stl")
    eng.add_mesh_stl(tmp_path / "tray.stl", position=(0.5, 0.5, 0.0), quaternion=q)
    return eng, pos, vel, 2e-5, funnel, tray


@pytest.mark.parametrize("engine", ["SHP", "SAP"])
def test_stl_hopper_bit_exact_vs_oracle(sdlib, orc, tmp_path, engine):
    """Two static STL meshes; sphere-triangle candidates from the static grid
    (SHP) or from sweep and prune along the meshes' longest extent (SAP)."""
    from stardust_gb300 import _abi
    eng, pos, vel, dt, funnel, tray = hopper_engine(sdlib, tmp_path, engine=getattr(_abi, "SD_ENGINE_" + engine))
    t, pa, c = eng.mesh()
    assert len(t) == 18 and len(np.unique(pa)) == 9
    assert np.allclose(t + np.float32(c), np.concatenate([funnel, tray]), atol=1e-6)  # the tray is back in place
    eng.prepare()
    eng.step(dt, 0)
    eng.sync()
    mesh = orc.make_mesh_frame(t, pa, eng.mesh_state())
    p = orc.params_checked(eng.config, pos[:, 3], dt, eng.params())
    n = len(pos)
    omg = orc.with_ids(np.zeros_like(pos), np.arange(n))
    steps = 4000
    op, ov, ow, _ = orc.run_full(p, eng.positions(), eng.velocities(), omg, steps, mesh=mesh)
    eng.step(dt, steps)
    eng.sync()
    assert eng.stats()["device_errors"] == 0
    assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
    assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
    # the spheres fell into the funnel and the outer ones were pushed inwards
    # by its walls: nobody is outside the funnel at its height
    q = eng.positions().astype(np.float64)
    assert q[:, 2].max() < 0.125
    half = 0.015 + (q[:, 2] - 0.06) / 0.08 * 0.045  # the funnel's inner half-width at each sphere's height
    inside = q[:, 2] > 0.06
    assert np.all(np.maximum(np.abs(q[inside, 0]), np.abs(q[inside, 1])) < half[inside])
    assert np.abs(eng.velocities()[:, :2]).max() > 1e-3  # deflected sideways by the sloped walls
    eng.close()
