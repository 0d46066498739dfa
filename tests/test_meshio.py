"""Mesh entities from STL files (host side, CPU only): the library's STL
reader (ASCII and binary) against files written by stardust_gb300.meshio,
its error handling, the smooth-face patch rule, placement by position and
quaternion, combining static meshes, and the JSON scene's "mesh" entity.
The reference reads STL through the third-party stl_reader header
(src/IO/mesh_loader.cpp:9-45) into DEMMesh (entity.hpp:64-93)."""
import json

import numpy as np
import pytest


def box_tris(lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
    """A closed box, 12 triangles, consistently wound (outward normals)."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float32)
    f = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4),
         (1, 2, 6), (1, 6, 5), (2, 3, 7), (2, 7, 6), (3, 0, 4), (3, 4, 7)]
    return v[np.array(f)]


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("binary", [True, False])
def test_stl_round_trip_is_exact(sdlib, tmp_path, binary):
    from stardust_gb300 import scenes
    tris, _ = scenes.drum_mesh(0.05, 0.04, 24, 5, 3, (0.1, 0.2, 0.3))
    rng = np.random.default_rng(0)
    tris = tris + rng.uniform(-1e-3, 1e-3, tris.shape).astype(np.float32)  # arbitrary float bits
    f = tmp_path / "m.stl"
    sdlib.write_stl(f, tris, binary=binary)
    back = sdlib.read_stl(f)
    assert back.shape == tris.shape and np.array_equal(bits(back), bits(tris))


def test_binary_stl_whose_header_says_solid(sdlib, tmp_path):
    tris = box_tris()
    f = tmp_path / "b.stl"
    sdlib.write_stl(f, tris, binary=True, name="solid cube exported as binary")
    assert f.read_bytes()[:5] == b"solid"
    assert np.array_equal(sdlib.read_stl(f), tris)


def test_ascii_stl_with_several_solids(sdlib, tmp_path):
    a, b = box_tris(), box_tris((2, 0, 0), (3, 1, 1))
    fa, fb = tmp_path / "a.stl", tmp_path / "b.stl"
    sdlib.write_stl(fa, a, binary=False, name="first")
    sdlib.write_stl(fb, b, binary=False, name="second")
    both = tmp_path / "both.stl"
    both.write_text(fa.read_text() + fb.read_text())
    assert np.array_equal(sdlib.read_stl(both), np.concatenate([a, b]))


@pytest.mark.parametrize("content, what", [
    (b"", "not an STL"),
    (b"solid x\n facet normal 0 0 1\n outer loop\n vertex 0 0 0\n vertex 1 0 0\n endloop\n endfacet\nendsolid x\n",
     "2 vertices"),
    (b"solid x\n facet normal 0 0 1\n outer loop\n vertex 0 0 0\n vertex 1 zero 0\n", "bad vertex"),
    (b"solid x\n facet normal 0 0 1\n outer loop\n vertex 0 0 0\n vertex 1 0 0\n vertex 0 1 0\n", "ends inside"),
    (b"hello world", "not an STL"),
    (b"\0" * 80 + np.uint32(3).tobytes() + b"\0" * 100, "not an STL"),  # binary, truncated
])
def test_stl_errors(sdlib, tmp_path, content, what):
    f = tmp_path / "bad.stl"
    f.write_bytes(content)
    with pytest.raises(sdlib.SdError) as e:
        sdlib.read_stl(f)
    assert what in str(e.value)


def test_stl_missing_file(sdlib, tmp_path):
    with pytest.raises(sdlib.SdError) as e:
        sdlib.read_stl(tmp_path / "nope.stl")
    assert "cannot read" in str(e.value)


def test_patches_box_drum_and_winding(sdlib):
    from stardust_gb300 import scenes
    box = box_tris()
    p = sdlib.mesh_patches(box, 30.0)
    assert len(np.unique(p)) == 6 and np.all(p[0::2] == p[1::2])  # two triangles per face
    assert list(p[0::2]) == [0, 1, 2, 3, 4, 5]  # numbered by first triangle
    # the constructed drum's own faces: side wall + two caps
    tris, patch = scenes.drum_mesh(0.5, 0.5, 128, 65, 8, (0.25, 0.5, 0.5))
    assert np.array_equal(sdlib.mesh_patches(tris, 30.0), patch)
    # flipping the winding of some triangles does not split a face
    flipped = box.copy()
    flipped[1::4] = flipped[1::4][:, ::-1]
    assert np.array_equal(sdlib.mesh_patches(flipped, 30.0), p)
    # a zero crease angle separates every triangle; 95 degrees joins the box
    assert len(np.unique(sdlib.mesh_patches(box, 0.0))) == 12
    assert len(np.unique(sdlib.mesh_patches(box, 95.0))) == 1


def test_add_mesh_stl_placement_and_static_combination(sdlib, tmp_path):
    box = box_tris((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)) * np.float32(0.1)
    f = tmp_path / "box.stl"
    sdlib.write_stl(f, box)
    eng = sdlib.DEMEngine()
    ang = 0.3
    q = (np.cos(ang / 2), 0.0, 0.0, np.sin(ang / 2))  # about z
    eng.add_mesh_stl(f, position=(1.0, 2.0, 3.0), quaternion=q)
    t, pa, c = eng.mesh()
    assert c == (0.0, 0.0, 0.0) and len(t) == 12
    R = np.array([[np.cos(ang), -np.sin(ang), 0], [np.sin(ang), np.cos(ang), 0], [0, 0, 1]])
    want = box.astype(np.float64) @ R.T + np.array([1.0, 2.0, 3.0])
    assert np.max(np.abs(t - want)) < 1e-6
    assert len(np.unique(pa)) == 6
    # a second static mesh is appended, its patches after the first's
    eng.add_mesh_stl(f, position=(0.0, 0.0, 1.0))
    t2, pa2, _ = eng.mesh()
    assert len(t2) == 24 and np.array_equal(t2[:12], t) and pa2[12:].min() == pa.max() + 1
    # a rotating mesh cannot join them
    with pytest.raises(sdlib.SdError) as e:
        eng.add_mesh_stl(f, centre=(0, 0, 0), axis=(1, 0, 0), omega=1.0)
    assert "rotating" in str(e.value)
    eng.close()


def test_json_mesh_entity(sdlib, tmp_path):
    box = box_tris((0.0, 0.0, 0.0), (0.5, 0.5, 0.5))
    (tmp_path / "meshes").mkdir()
    sdlib.write_stl(tmp_path / "meshes" / "bin.stl", box)
    scene = {"scene": {"box": {"lo": [-1, -1, -1], "hi": [2, 2, 2]}, "walls": 0, "cell": 0.05,
                       "entities": [
                           {"type": "mesh", "file": "meshes/bin.stl", "position": [0.1, 0, 0],
                            "quaternion": [1, 0, 0, 0], "patch_angle": 20},
                           {"type": "generic", "position": [0.25, 0.25, 0.7], "size": 0.04, "mass": 0.01}]}}
    f = tmp_path / "scene.json"
    f.write_text(json.dumps(scene))
    eng = sdlib.DEMEngine()
    eng.load_scene_json(f)
    t, pa, c = eng.mesh()
    assert len(t) == 12 and eng.n == 1
    assert np.array_equal(t, box + np.float32([0.1, 0, 0]))
    eng.close()
    # a rotating mesh entity
    scene["scene"]["entities"][0]["rotation"] = {"centre": [0.25, 0.25, 0.25], "axis": [0, 0, 1], "omega": 2.0}
    f.write_text(json.dumps(scene))
    eng = sdlib.DEMEngine()
    eng.load_scene_json(f)
    t, pa, c = eng.mesh()
    assert c == pytest.approx((0.25, 0.25, 0.25))
    eng.close()
    for bad, what in (({"type": "mesh"}, "file"), ({"type": "mesh", "file": "none.stl"}, "cannot read"),
                      ({"type": "mesh", "file": "meshes/bin.stl", "colour": 1}, "colour"),
                      ({"type": "mesh", "file": "meshes/bin.stl", "quaternion": [1, 0, 0]}, "quaternion"),
                      ({"type": "mesh", "file": "meshes/bin.stl", "patch_angle": 200}, "patch_angle")):
        scene["scene"]["entities"] = [bad]
        f.write_text(json.dumps(scene))
        eng = sdlib.DEMEngine()
        with pytest.raises(sdlib.SdError) as e:
            eng.load_scene_json(f)
        assert what in str(e.value)
        eng.close()
