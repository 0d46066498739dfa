"""The oracle derives the step's parameters itself (grid, cell_z, damping)
and checks them against the engine's (sd_engine_params), so a wrong
derivation in the library is caught instead of copied.  Also: the oracle's
copy of the seeded scene builders draws the same spheres as the library's.
Host-only calls: no GPU."""
import numpy as np
import pytest


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def engine_params(sdlib, cfg, pos, vel):
    eng = sdlib.DEMEngine(cfg)
    eng.add_spheres(pos, vel)
    ep = eng.params()
    eng.close()
    return ep


def test_scene_builders_match_the_library(sdlib, orc):
    from stardust_gb300 import scenes
    a = scenes.settling_rsa(20_000, box=scenes.scaled_box(20_000), seed=4)
    b = scenes.settling_rsa(20_000, box=scenes.scaled_box(20_000), seed=4, rsa=orc.scene_rsa)
    assert np.array_equal(bits(a[0]), bits(b[0])) and np.array_equal(bits(a[1]), bits(b[1])) and a[4] == b[4]
    a = scenes.box_lattice(16, seed=0)
    b = scenes.box_lattice(16, seed=0, lattice=orc.scene_lattice)
    assert np.array_equal(bits(a[0]), bits(b[0])) and np.array_equal(bits(a[1]), bits(b[1]))


def configs():
    from stardust_gb300 import EngineConfig, scenes
    out = []
    pos, vel, cfg, dt = scenes.box_lattice(16, seed=0)
    out.append(("lattice 4096", pos, vel, cfg, dt))
    for n in (4096, 20_000):
        pos, vel, cfg, dt, _ = scenes.settling_rsa(n, box=scenes.scaled_box(n), seed=0)
        out.append((f"settling {n}", pos, vel, cfg, dt))
    # the 1,048,576-sphere box's grid (cell 0.02 in 1 x 1 x 2 m), sparsely filled
    pos, vel, cfg, dt, _ = scenes.settling_rsa(2000, box=(1.0, 1.0, 2.0), seed=0)
    out.append(("settling grid 50x50x100", pos, vel, cfg, dt))
    rng = np.random.default_rng(1)
    pos = np.zeros((500, 4), np.float32)
    pos[:, :3] = rng.uniform(0.1, 0.6, (500, 3))
    pos[:, 3] = rng.uniform(0.002, 0.0071, 500)
    vel = np.zeros_like(pos)
    vel[:, 3] = 1e-3
    # a cell that does not divide the box, another restitution, the domain
    # in place of a box, open faces
    out.append(("odd cell", pos, vel, EngineConfig(box_lo=(-0.05, 0.0, 0.1), box_hi=(0.7, 0.66, 0.73), cell=0.0173,
                                                   restitution=0.8, kn=3e4, mu=0.1, walls=0x2B), 1e-5))
    out.append(("domain", pos, vel, EngineConfig(domain=0.75, restitution=0.3), 2e-5))
    out.append(("auto cell", pos, vel, EngineConfig(box_lo=(0.0, 0.0, 0.0), box_hi=(0.8, 0.8, 0.8)), 1e-5))
    return out


@pytest.mark.parametrize("k", range(7))
def test_engine_parameters_equal_the_oracles(sdlib, orc, k):
    name, pos, vel, cfg, dt = configs()[k]
    ep = engine_params(sdlib, cfg, pos, vel)
    p = orc.params_checked(cfg, pos[:, 3], dt, ep)
    assert p.nx * p.ny * p.nz == ep["dims"][0] * ep["dims"][1] * ep["dims"][2]


@pytest.mark.parametrize("z_div", [1, 2, 4, 8])
def test_engine_parameters_under_a_fixed_z_split(sdlib, orc, z_div):
    from stardust_gb300 import _abi, scenes
    old = _abi.tune_get("z_div")
    try:
        _abi.tune_set("z_div", z_div)
        pos, vel, cfg, dt, _ = scenes.settling_rsa(20_000, box=scenes.scaled_box(20_000), seed=0)
        ep = engine_params(sdlib, cfg, pos, vel)
    finally:
        _abi.tune_set("z_div", old)
    assert ep["z_div"] == z_div
    orc.params_checked(cfg, pos[:, 3], dt, ep, z_div=z_div)


def test_a_planted_difference_is_reported(sdlib, orc):
    """The check fails when the oracle's inputs differ from the engine's:
    another restitution (damping), another cell edge (grid)."""
    import dataclasses
    name, pos, vel, cfg, dt = configs()[0]
    ep = engine_params(sdlib, cfg, pos, vel)
    with pytest.raises(AssertionError, match="damp"):
        orc.params_checked(dataclasses.replace(cfg, restitution=0.51), pos[:, 3], dt, ep)
    with pytest.raises(AssertionError, match="dims"):
        orc.params_checked(dataclasses.replace(cfg, cell=0.0213), pos[:, 3], dt, ep)
