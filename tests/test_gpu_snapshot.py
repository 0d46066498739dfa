"""Headless snapshots (sd_engine_write_snapshot) read back against the
engine's own state: CSV and legacy binary VTK, with contact pairs and the
mesh at its current pose.  The reference draws with OpenGL and writes no
files (src/graphics/renderer.cpp:15-22, 146-147)."""
import numpy as np
import pytest


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def read_vtk(path):
    """Minimal reader of the legacy binary POLYDATA this library writes."""
    data = open(path, "rb").read()
    pos = 0
    out = {"cells": {}, "scalars": {}, "vectors": {}}

    def line():
        nonlocal pos
        end = data.index(b"\n", pos)
        s = data[pos:end].decode()
        pos = end + 1
        return s

    def block(count, dtype):
        nonlocal pos
        a = np.frombuffer(data, dtype=dtype, count=count, offset=pos)
        pos += a.nbytes
        return a

    assert line().startswith("# vtk DataFile")
    out["title"] = line()
    assert line() == "BINARY" and line() == "DATASET POLYDATA"
    npts = 0
    while pos < len(data):
        s = line()
        if not s:
            continue
        w = s.split()
        if w[0] == "POINTS":
            npts = int(w[1])
            out["points"] = block(3 * npts, ">f4").reshape(-1, 3)
        elif w[0] in ("VERTICES", "LINES", "POLYGONS"):
            out["cells"][w[0]] = block(int(w[2]), ">i4")
        elif w[0] == "POINT_DATA":
            assert int(w[1]) == npts
        elif w[0] == "SCALARS":
            assert line() == "LOOKUP_TABLE default"
            out["scalars"][w[1]] = block(npts, ">f4" if w[2] == "float" else ">i4")
        elif w[0] == "VECTORS":
            out["vectors"][w[1]] = block(3 * npts, ">f4").reshape(-1, 3)
        else:
            raise AssertionError(s)
    return out


def test_snapshot_needs_a_prepared_engine(sdlib, tmp_path):
    eng = sdlib.DEMEngine()
    eng.add_spheres(np.array([[0.5, 0.5, 0.5, 0.01]], np.float32), np.array([[0, 0, 0, 1e-3]], np.float32))
    with pytest.raises(sdlib.SdError):
        eng.write_snapshot(tmp_path / "s.vtk")
    with pytest.raises(ValueError):
        eng.write_snapshot(tmp_path / "s.xyz", fmt="xyz")
    eng.close()


@pytest.mark.gpu
def test_csv_and_vtk_snapshots_are_the_state(sdlib, tmp_path):
    from stardust_gb300 import scenes
    pos, vel, cfg, dt, phi = scenes.settling_rsa(5000, box=scenes.scaled_box(5000), seed=3)
    pos = pos.copy()
    pos[:, 3] *= 1.25  # overlaps: contact pairs to write
    cfg.cell = float(2 * pos[:, 3].max())
    omega = np.zeros_like(pos)
    omega[:, :3] = np.random.default_rng(0).uniform(-5, 5, (len(pos), 3))
    eng = sdlib.DEMEngine(cfg)
    eng.add_spheres(pos, vel, omega)
    eng.prepare()
    eng.step(dt, 7)
    eng.sync()
    p, v, w, pairs = eng.positions(), eng.velocities(), eng.omegas(), eng.pairs()
    assert len(pairs) > 100
    eng.write_snapshot(tmp_path / "s.csv", fmt="csv", contacts=True)
    eng.write_snapshot(tmp_path / "s.vtk", fmt="vtk", contacts=True)
    eng.close()
    t = np.loadtxt(tmp_path / "s.csv", delimiter=",", skiprows=1, dtype=np.float64)
    assert np.array_equal(t[:, 0], np.arange(len(p)))
    assert np.array_equal(bits(t[:, 1:5].astype(np.float32)), bits(p))
    assert np.array_equal(bits(t[:, 5:9].astype(np.float32)), bits(v))
    assert np.array_equal(bits(t[:, 9:12].astype(np.float32)), bits(w[:, :3]))
    c = np.loadtxt(tmp_path / "s.csv.contacts.csv", delimiter=",", skiprows=1, dtype=np.uint64).reshape(-1, 2)
    assert np.array_equal((c[:, 0] << np.uint64(32)) | c[:, 1], pairs)
    d = read_vtk(tmp_path / "s.vtk")
    n = len(p)
    assert np.array_equal(bits(d["points"]), bits(p[:, :3]))
    assert np.array_equal(d["cells"]["VERTICES"].reshape(-1, 2), np.stack([np.ones(n), np.arange(n)], 1))
    lines = d["cells"]["LINES"].reshape(-1, 3).astype(np.uint64)
    assert np.all(lines[:, 0] == 2) and np.array_equal((lines[:, 1] << np.uint64(32)) | lines[:, 2], pairs)
    assert np.array_equal(bits(d["scalars"]["radius"]), bits(p[:, 3]))
    assert np.array_equal(bits(d["scalars"]["mass"]), bits(v[:, 3]))
    assert np.array_equal(d["scalars"]["id"], np.arange(n))
    assert np.array_equal(bits(d["vectors"]["velocity"]), bits(v[:, :3]))
    assert np.array_equal(bits(d["vectors"]["spin"]), bits(w[:, :3]))
    assert "step 7" in d["title"]


@pytest.mark.gpu
def test_vtk_snapshot_carries_the_turning_mesh(sdlib, tmp_path):
    from stardust_gb300 import scenes
    d = scenes.drum_scene(n_spheres=650, radius=0.04, length=0.04, n_around=24, n_along=6, n_rings=3,
                          r_range=(0.002, 0.0028), omega=20.0, seed=0)
    eng = sdlib.DEMEngine(d["cfg"])
    scenes.add_drum_scene(eng, d)
    eng.prepare()
    eng.step(d["dt"], 500)
    eng.sync()
    eng.write_snapshot(tmp_path / "drum.vtk", mesh=True)
    frame, patch, centre = eng.mesh()
    st = eng.mesh_state()
    n = eng.n
    p = eng.positions()
    eng.close()
    v = read_vtk(tmp_path / "drum.vtk")
    nt = len(frame)
    assert len(v["points"]) == n + 3 * nt
    assert np.array_equal(bits(v["points"][:n]), bits(p[:, :3]))
    poly = v["cells"]["POLYGONS"].reshape(-1, 4)
    assert len(poly) == nt and np.all(poly[:, 0] == 3) and np.array_equal(poly[:, 1:].ravel(), n + np.arange(3 * nt))
    R = st[:9].astype(np.float64).reshape(3, 3)
    want = frame.reshape(-1, 3).astype(np.float64) @ R.T + st[9:12].astype(np.float64)
    assert np.max(np.abs(v["points"][n:] - want)) < 1e-6
    # 500 steps of 2e-6 s at 20 rad/s turn the mesh by 0.02 rad: not its time-0 placement
    assert np.max(np.abs(v["points"][n:] - (frame.reshape(-1, 3) + np.float32(centre)))) > 1e-4
    assert np.all(v["scalars"]["id"][n:] == -1)
