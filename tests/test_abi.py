"""The C-ABI library loads without a GPU, exports every declared symbol, and
its host-only entry points (config, scene loading, generators, parameter
derivation, error reporting) behave as documented."""
import ctypes as C
import json
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    names = []
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*sd_status\s+(sd_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(sdlib):
    names = declared_functions()
    assert len(names) >= 25
    lib = C.CDLL(str(sdlib._abi.LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_every_declared_symbol_has_a_binding(sdlib):
    assert set(declared_functions()) <= set(sdlib._abi.SIGNATURES)


def test_config_default_and_bad_struct_size(sdlib):
    c = sdlib._abi.SdConfig()
    sdlib._abi.call("sd_config_default", C.byref(c))
    assert c.struct_size == C.sizeof(sdlib._abi.SdConfig)
    assert c.kn == pytest.approx(1e5) and c.restitution == pytest.approx(0.5) and c.mu == pytest.approx(0.3)
    c.struct_size = 7
    h = C.c_void_p()
    st = sdlib.lib().sd_engine_create(C.byref(c), C.byref(h))
    assert st == sdlib._abi.SD_ERR_INVALID_ARG
    assert "struct_size" in sdlib._abi.last_error()


def test_cpu_device_is_rejected(sdlib):
    cfg = sdlib.EngineConfig(device=sdlib._abi.SD_DEVICE_CPU)
    with pytest.raises(sdlib.SdError) as e:
        sdlib.DEMEngine(cfg)
    assert e.value.status == sdlib._abi.SD_ERR_UNSUPPORTED


def test_add_spheres_validates(sdlib):
    eng = sdlib.DEMEngine()
    with pytest.raises(sdlib.SdError) as e:
        eng.add_spheres(np.array([[0.5, 0.5, 0.5, 0.0]], np.float32), np.array([[0, 0, 0, 1.0]], np.float32))
    assert e.value.status == sdlib._abi.SD_ERR_INVALID_ARG
    with pytest.raises(sdlib.SdError):
        eng.add_spheres(np.array([[np.nan, 0.5, 0.5, 0.1]], np.float32), np.array([[0, 0, 0, 1.0]], np.float32))
    eng.close()


def test_cube_particle_is_a_clump(sdlib):
    """DEMParticle(grid_resolution > 1) (entity.cpp:9-59): grid_resolution^3
    spheres spaced size / floor(size/diameter)^2, one rigid body."""
    eng = sdlib.DEMEngine()
    eng.add(2, 0.2, 0.1, 3.0, (0.5, 0.5, 0.5), (0, 0, 0))
    st = eng.stats()
    assert st["n_spheres"] == 8 and st["n_bodies"] == 1
    eng.add(1, 0.1, 0.1, 3.0, (0.2, 0.2, 0.2), (0, 0, 0))
    st = eng.stats()
    assert st["n_spheres"] == 9 and st["n_bodies"] == 1
    with pytest.raises(sdlib.SdError) as e:
        eng.add(2, 0.05, 0.1, 3.0, (0.5, 0.5, 0.5), (0, 0, 0))
    assert e.value.status == sdlib._abi.SD_ERR_INVALID_ARG
    eng.close()


def test_add_clump_validates(sdlib):
    eng = sdlib.DEMEngine()
    rel = np.array([[0.05, 0, 0, 0.05], [-0.05, 0, 0, 0.05]], np.float32)
    with pytest.raises(sdlib.SdError) as e:
        eng.add_clump(rel, 0.0, (0.5, 0.5, 0.5))
    assert e.value.status == sdlib._abi.SD_ERR_INVALID_ARG
    with pytest.raises(sdlib.SdError) as e:
        eng.add_clump(np.array([[0, 0, 0, -1.0]], np.float32), 1.0, (0.5, 0.5, 0.5))
    assert e.value.status == sdlib._abi.SD_ERR_INVALID_ARG
    eng.add_clump(rel, 1.0, (0.5, 0.5, 0.5), (0, 0, 1.0), (0, 2.0, 0))
    assert eng.stats()["n_bodies"] == 1 and eng.n == 2
    eng.close()


def test_params_derivation(sdlib):
    from stardust_gb300 import scenes
    pos, vel, cfg, dt = scenes.box_lattice(n_side=4)
    eng = sdlib.DEMEngine(cfg)
    eng.add_spheres(pos, vel)
    p = eng.params()
    # 32^3 cells, z split 4x finer: 17-bit keys still sort in 2 passes
    assert p["z_div"] == 4 and p["dims"] == (32, 32, 128)
    assert p["cell"] == pytest.approx(0.02) and p["cell_z"] == pytest.approx(0.005)
    # gamma_n = damp sqrt(m_eff); damp = 2 beta sqrt(kn), beta = -ln e / sqrt(pi^2 + ln^2 e)
    le = np.log(0.5)
    beta = -le / np.sqrt(np.pi ** 2 + le ** 2)
    assert p["damp"] == pytest.approx(2 * beta * np.sqrt(1e5), rel=1e-6)
    eng.close()


def test_cell_smaller_than_diameter_rejected(sdlib):
    cfg = sdlib.EngineConfig(box_hi=(1, 1, 1), cell=0.01)
    eng = sdlib.DEMEngine(cfg)
    eng.add_spheres(np.array([[0.5, 0.5, 0.5, 0.02]], np.float32), np.array([[0, 0, 0, 1.0]], np.float32))
    with pytest.raises(sdlib.SdError) as e:
        eng.params()
    assert e.value.status == sdlib._abi.SD_ERR_INVALID_ARG
    eng.close()


def test_reference_scene_json_loads(sdlib, tmp_path):
    # the schema of setup/star_test.json: scene.domain, entities[], gravity
    scene = {"scene": {"domain": 4, "entities": [
        {"type": "generic", "position": [0.5, 0.5, 0.5], "size": 0.15, "mass": 3, "velocity": [0, 0, 0]},
        {"type": "generic", "position": [1, 1, 1], "size": 0.15, "mass": 3, "velocity": [0, 0, 0]}],
        "gravity": 9.81}}
    f = tmp_path / "star_test.json"
    f.write_text(json.dumps(scene, indent=4))
    eng = sdlib.DEMEngine()
    eng.load_scene_json(f)
    assert eng.n == 2
    p = eng.params()
    assert p["hi"] == pytest.approx((4, 4, 4)) and p["lo"] == pytest.approx((0, 0, 0))
    assert p["gravity"] == pytest.approx((0, 0, -9.81))
    assert p["cell"] == pytest.approx(0.15)  # 2 x radius (diameter = size)
    eng.close()


def test_scene_json_cube_entities(sdlib, tmp_path):
    # a generic entity with grid_resolution > 1 is a DEMParticle cube clump;
    # sphere ids follow the file order
    scene = {"scene": {"domain": 2, "entities": [
        {"type": "generic", "position": [0.5, 0.5, 0.5], "size": 0.1, "mass": 1},
        {"type": "generic", "position": [1, 1, 1], "size": 0.2, "diameter": 0.1, "grid_resolution": 2, "mass": 3},
        {"type": "generic", "position": [1.5, 1.5, 1.5], "size": 0.1, "mass": 1}]}}
    f = tmp_path / "cubes.json"
    f.write_text(json.dumps(scene))
    eng = sdlib.DEMEngine()
    eng.load_scene_json(f)
    st = eng.stats()
    assert st["n_spheres"] == 10 and st["n_bodies"] == 1 and eng.n == 10
    eng.close()
    bad = {"scene": {"entities": [{"type": "generic", "position": [0, 0, 0], "size": 0.1, "mass": 1,
                                   "grid_resolution": 2.5}]}}
    g = tmp_path / "bad_cube.json"
    g.write_text(json.dumps(bad))
    e2 = sdlib.DEMEngine()
    with pytest.raises(sdlib.SdError) as e:
        e2.load_scene_json(g)
    assert e.value.status == sdlib._abi.SD_ERR_JSON and "grid_resolution" in str(e.value)
    e2.close()


@pytest.mark.parametrize("knob, box, want", [
    (0, (1.0, 1.0, 2.0), 4),    # 50 x 50 x 100: 18-bit keys -> 20-bit, 2 passes (10 + 10 bits)
    (0, (0.5, 0.5, 0.5), 4),    # 25^3: 14 bits -> 16, 2 passes
    (0, (1.4, 1.4, 1.4), 2),    # 70^3: 19 bits -> 20 at x2 (21 at x4: a third pass)
    (0, (1.8, 1.8, 1.8), 1),    # 90^3: 20 bits; x2 would need 21 bits and a third pass
    (0, (5.0, 5.0, 5.0), 1),    # 250^3: 24-bit keys, no split (measured slower on the drum)
    (1, (1.0, 1.0, 2.0), 1),
    (8, (1.0, 1.0, 2.0), 8),
])
def test_z_div_rule_and_knob(sdlib, knob, box, want):
    from stardust_gb300 import _abi
    old = _abi.tune_get("z_div")
    try:
        _abi.tune_set("z_div", knob)
        cfg = sdlib.EngineConfig(box_lo=(0, 0, 0), box_hi=box, walls=0x3F, cell=0.02, kn=1e5, restitution=0.5,
                                 mu=0.3, gravity=(0.0, 0.0, -9.81))
        eng = sdlib.DEMEngine(cfg)
        eng.add_spheres(np.array([[0.5, 0.5, 0.5, 0.01]], np.float32), np.array([[0, 0, 0, 1e-3]], np.float32))
        p = eng.params()
        nz = int(np.ceil(box[2] / np.float32(0.02) * (1 - 1e-6)))
        assert p["z_div"] == want and p["dims"][2] == nz * want
        assert p["cell_z"] == np.float32(np.float32(0.02) / np.float32(want))
        eng.close()
    finally:
        _abi.tune_set("z_div", old)
    with pytest.raises(Exception):
        _abi.tune_set("z_div", 3)


def test_scene_json_extensions_and_errors(sdlib, tmp_path):
    ok = {"scene": {"box": {"lo": [0, 0, 0], "hi": [1, 1, 2]}, "walls": 63, "cell": 0.05,
                    "material": {"kn": 2e5, "restitution": 0.8, "mu": 0.1},
                    "spheres": [{"position": [0.5, 0.5, 0.5], "radius": 0.01, "mass": 0.001}]}}
    f = tmp_path / "ok.json"
    f.write_text(json.dumps(ok))
    eng = sdlib.DEMEngine()
    eng.load_scene_json(f)
    p = eng.params()
    assert p["dims"] == (20, 20, 160) and p["z_div"] == 4 and p["kn"] == pytest.approx(2e5) and p["mu"] == pytest.approx(0.1)
    eng.close()
    for bad, what in (({"scene": {"domain": 1, "colour": 3}}, "colour"),
                      ({"scene": {"entities": [{"type": "cloud", "position": [0, 0, 0], "size": 1, "mass": 1}]}}, "generic"),
                      ({"scene": {"entities": [{"type": "generic", "position": [0, 0], "size": 1, "mass": 1}]}}, "position"),
                      ({"nope": {}}, "nope")):
        g = tmp_path / "bad.json"
        g.write_text(json.dumps(bad))
        e2 = sdlib.DEMEngine()
        with pytest.raises(sdlib.SdError) as e:
            e2.load_scene_json(g)
        assert e.value.status == sdlib._abi.SD_ERR_JSON and what in str(e.value)
        e2.close()
    g = tmp_path / "broken.json"
    g.write_text('{"scene": {"domain": 1,}')
    e3 = sdlib.DEMEngine()
    with pytest.raises(sdlib.SdError) as e:
        e3.load_scene_json(g)
    assert e.value.status == sdlib._abi.SD_ERR_JSON
    with pytest.raises(sdlib.SdError) as e:
        e3.load_scene_json(tmp_path / "missing.json")
    assert e.value.status == sdlib._abi.SD_ERR_IO
    e3.close()


def test_state_calls_before_prepare_are_errors(sdlib):
    eng = sdlib.DEMEngine()
    eng.add_spheres(np.array([[0.5, 0.5, 0.5, 0.1]], np.float32), np.array([[0, 0, 0, 1.0]], np.float32))
    for fn in (lambda: eng.step(1e-5, 1), lambda: eng.positions(), lambda: eng.pairs()):
        with pytest.raises(sdlib.SdError) as e:
            fn()
        assert e.value.status == sdlib._abi.SD_ERR_STATE
    eng.close()


def test_generators_are_seeded(sdlib):
    from stardust_gb300 import scenes
    a = scenes.box_lattice(n_side=6, seed=3)[0]
    b = scenes.box_lattice(n_side=6, seed=3)[0]
    c = scenes.box_lattice(n_side=6, seed=4)[0]
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    # jitter bound and spacing of the lattice
    assert np.all(np.abs(np.diff(np.sort(np.unique(np.round(a[:, 0], 3))))) > 0.02)


def test_rsa_is_non_overlapping(sdlib):
    from stardust_gb300 import scenes
    n = 3000
    pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=scenes.scaled_box(n), seed=5)
    assert 0.30 < phi < 0.40
    d = pos[:, None, :3].astype(np.float64) - pos[None, :, :3]
    dist = np.sqrt((d ** 2).sum(-1))
    rs = pos[:, None, 3].astype(np.float64) + pos[None, :, 3]
    np.fill_diagonal(dist, 1e9)
    assert np.all(dist >= rs * (1 - 1e-6))
    lo, hi = np.array(cfg.box_lo), np.array(cfg.box_hi)
    assert np.all(pos[:, :3] - pos[:, 3:4] >= lo - 1e-7) and np.all(pos[:, :3] + pos[:, 3:4] <= hi + 1e-7)
    assert np.all((pos[:, 3] >= 0.0025) & (pos[:, 3] <= 0.01))
    assert np.allclose(vel[:, 3], scenes.DENSITY * 4 / 3 * np.pi * pos[:, 3].astype(np.float64) ** 3, rtol=1e-6)


def test_batch_api_rules(sdlib):
    import numpy as np
    pos = np.array([[0.5, 0.5, 0.5, 0.01]], np.float32)
    vel = np.array([[0, 0, 0, 1e-3]], np.float32)
    eng = sdlib.DEMEngine()
    eng.add_scene(pos, vel, (0, 0, 0), (1, 1, 1))
    with pytest.raises(sdlib.SdError) as e:
        eng.add_spheres(pos, vel)
    assert e.value.status == sdlib._abi.SD_ERR_STATE
    with pytest.raises(sdlib.SdError) as e:
        eng.add_scene(pos, vel, (0, 0, 0), (1, 0, 1))
    assert e.value.status == sdlib._abi.SD_ERR_INVALID_ARG
    eng.add_scene(pos, vel, (0, 0, 0), (2, 2, 2))
    assert eng.stats()["n_spheres"] == 2
    eng.close()
    e2 = sdlib.DEMEngine()
    e2.add_spheres(pos, vel)
    with pytest.raises(sdlib.SdError) as e:
        e2.add_scene(pos, vel, (0, 0, 0), (1, 1, 1))
    assert e.value.status == sdlib._abi.SD_ERR_STATE
    e2.close()


def test_resort_max_knob(sdlib):
    from stardust_gb300 import _abi
    old = _abi.tune_get("resort_max")
    assert old == 1024
    try:
        for v in (0, 1, 2, 256, 1024):
            _abi.tune_set("resort_max", v)
            assert _abi.tune_get("resort_max") == v
        for v in (-1, 3, 1000, 2048, 4096):
            with pytest.raises(Exception):
                _abi.tune_set("resort_max", v)
    finally:
        _abi.tune_set("resort_max", old)


def test_pair_lists_knob(sdlib):
    from stardust_gb300 import _abi
    old = _abi.tune_get("pair_lists")
    assert old == 2
    try:
        for v in (0, 1, 2):
            _abi.tune_set("pair_lists", v)
            assert _abi.tune_get("pair_lists") == v
        with pytest.raises(Exception):
            _abi.tune_set("pair_lists", 3)
    finally:
        _abi.tune_set("pair_lists", old)


@pytest.mark.parametrize("cname,pyname", [("sd_config", "SdConfig"), ("sd_stats", "SdStats"),
                                          ("sd_params", "SdParams")])
def test_struct_layouts_match_the_header(tmp_path, cname, pyname):
    """The ctypes mirrors of the C structs have the header's size and every
    field at the header's offset (compiled with the host C compiler)."""
    import shutil
    import subprocess
    from stardust_gb300 import _abi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    py = getattr(_abi, pyname)
    fields = [f[0] for f in py._fields_]
    lines = [f'printf("%zu\\n", sizeof({cname}));'] + [f'printf("%zu\\n", offsetof({cname}, {f}));' for f in fields]
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "stardust.h"\nint main(void) {\n'
                   + "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert out[0] == C.sizeof(py)
    assert out[1:] == [getattr(py, f).offset for f in fields]


def test_skin_knob(sdlib):
    from stardust_gb300 import _abi
    old = _abi.tune_get("skin_um")
    assert old == 50  # the default
    try:
        _abi.tune_set("skin_um", 500)
        assert _abi.tune_get("skin_um") == 500
        for v in (-1, 100001):
            with pytest.raises(Exception):
                _abi.tune_set("skin_um", v)
    finally:
        _abi.tune_set("skin_um", old)


def test_hull_blocks_knob(sdlib):
    from stardust_gb300 import _abi
    old = _abi.tune_get("hull_blocks")
    assert old == 4
    try:
        _abi.tune_set("hull_blocks", 3)
        assert _abi.tune_get("hull_blocks") == 3
        for v in (0, 2, 5):
            with pytest.raises(Exception):
                _abi.tune_set("hull_blocks", v)
    finally:
        _abi.tune_set("hull_blocks", old)


def test_lbvh_rebuild_knob(sdlib):
    from stardust_gb300 import _abi
    old = _abi.tune_get("lbvh_rebuild")
    assert old == 16
    try:
        for v in (1, 7, 4096):
            _abi.tune_set("lbvh_rebuild", v)
            assert _abi.tune_get("lbvh_rebuild") == v
        for v in (0, -1, 4097):
            with pytest.raises(Exception):
                _abi.tune_set("lbvh_rebuild", v)
    finally:
        _abi.tune_set("lbvh_rebuild", old)


def test_listed_blocks_knob(sdlib):
    from stardust_gb300 import _abi
    old = _abi.tune_get("listed_blocks")
    assert old == 5
    try:
        for v in (4, 5, 6, 8):
            _abi.tune_set("listed_blocks", v)
            assert _abi.tune_get("listed_blocks") == v
        for v in (0, 3, 7, 9):
            with pytest.raises(Exception):
                _abi.tune_set("listed_blocks", v)
    finally:
        _abi.tune_set("listed_blocks", old)
