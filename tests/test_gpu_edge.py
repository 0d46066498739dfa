"""Edge cases of the sphere step on the GPU: an empty engine, a single
sphere, spheres outside the box (their cells clamp, the walls push them
back), pairs exactly at contact distance and coincident centres (neither
is a contact: the test is strict and a zero distance has no normal), all
against the oracle where it applies."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def cfg_box(sd, edge=1.0, cell=0.02, walls=0x3F, gravity=(0.0, 0.0, -9.81)):
    return sd.EngineConfig(box_lo=(0.0, 0.0, 0.0), box_hi=(edge, edge, edge), walls=walls, cell=cell, kn=1e5,
                           restitution=0.5, mu=0.3, gravity=gravity)


def test_empty_engine_steps(sdlib, tmp_path):
    eng = sdlib.DEMEngine(cfg_box(sdlib))
    eng.prepare()
    eng.step(1e-5, 10)
    eng.sync()
    st = eng.stats()
    assert st["n_spheres"] == 0 and st["steps"] == 10 and st["device_errors"] == 0
    assert len(eng.pairs()) == 0 and eng.positions().shape == (0, 4)
    eng.write_snapshot(tmp_path / "empty.vtk")
    eng.close()


def test_single_sphere_comes_to_rest_on_the_floor(sdlib, orc):
    eng = sdlib.DEMEngine(cfg_box(sdlib))
    pos = np.array([[0.5, 0.5, 0.03, 0.01]], np.float32)  # a 2 cm drop: the bounces die out within 0.5 s
    vel = np.array([[0.0, 0.0, 0.0, 1e-3]], np.float32)
    eng.add_spheres(pos, vel)
    eng.prepare()
    p = orc.params_checked(eng.config, pos[:, 3], 1e-5, eng.params())
    op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), [0]), 50000)
    eng.step(1e-5, 50000)
    eng.sync()
    assert np.array_equal(bits(eng.positions()), bits(op))
    z = float(eng.positions()[0, 2])
    assert abs(z - 0.01) < 1e-3 and abs(float(eng.velocities()[0, 2])) < 0.05
    eng.close()


def test_spheres_outside_the_box(sdlib, orc):
    """Centres beyond every face (and NaN-free far outside): their keys clamp
    to the edge cells; the walls push them in; bit-exact with the oracle."""
    rng = np.random.default_rng(2)
    pos = np.zeros((400, 4), np.float32)
    pos[:, :3] = rng.uniform(-0.05, 1.05, (400, 3))
    pos[:8, :3] = [[-0.3, 0.5, 0.5], [1.3, 0.5, 0.5], [0.5, -0.3, 0.5], [0.5, 1.3, 0.5], [0.5, 0.5, -0.3],
                   [0.5, 0.5, 1.3], [-5.0, -5.0, -5.0], [7.0, 7.0, 7.0]]
    pos[:, 3] = 0.01
    vel = np.zeros_like(pos)
    vel[:, 3] = 1e-3
    eng = sdlib.DEMEngine(cfg_box(sdlib))
    eng.add_spheres(pos, vel)
    eng.prepare()
    p = orc.params_checked(eng.config, pos[:, 3], 1e-5, eng.params())
    op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(len(pos))), 50)
    eng.step(1e-5, 50)
    eng.sync()
    assert eng.stats()["device_errors"] == 0
    assert np.array_equal(bits(eng.positions()), bits(orc.unsort(op, ow)))
    assert np.array_equal(bits(eng.velocities()), bits(orc.unsort(ov, ow)))
    assert np.all(np.isfinite(eng.positions())) and np.all(np.isfinite(eng.velocities()))
    eng.close()


def test_exact_contact_distance_and_coincident_centres(sdlib):
    """d == r_i + r_j is not a contact (the test is d^2 < (r_i + r_j)^2);
    two spheres with the same centre are not one either (no normal).
    Coordinates are exact binary fractions, so the distances are exact."""
    r = 0.125
    pos = np.array([[0.25, 0.25, 0.25, r], [0.5, 0.25, 0.25, r],                # touching exactly
                    [0.25, 0.75, 0.75, r], [0.25, 0.75, 0.75, r],               # coincident
                    [0.75, 0.75, 0.25, r], [0.75, 0.5 + 2 ** -10, 0.25, r]],    # overlapping by 2^-10
                   np.float32)
    vel = np.zeros_like(pos)
    vel[:, 3] = 1e-3
    eng = sdlib.DEMEngine(cfg_box(sdlib, walls=0, gravity=(0.0, 0.0, 0.0), cell=0.25))
    eng.add_spheres(pos, vel)
    eng.prepare()
    assert eng.pairs().tolist() == [(4 << 32) | 5]
    eng.step(1e-5, 1)
    eng.sync()
    v = eng.velocities()
    assert np.all(v[:4, :3] == 0) and v[4, 1] > 0 > v[5, 1]
    eng.close()
