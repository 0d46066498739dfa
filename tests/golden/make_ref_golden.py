"""Writes golden vectors from the reference's own kernels.

Runs on a machine with a GPU: loads the reference kernels that
``oracle/ref_build.py`` compiled from the reference sources
(``oracle/_ref/*.cubin``) through ``oracle/_ref/libref_harness.so`` and runs
them on seeded inputs:

* ``ref_hash_<case>.npz`` -- constructCollisionListCUDA
  (src/engine/cuda/sh_collision_detection.cu:27-127): positions, sizes, cell
  size -> the 9n (cell, sphere) words and the valid-entry count;
* ``ref_traverse_<case>.npz`` -- tranverseCollisionListCUDA +
  resolveCollisionsCUDA (collision_resolution.cu:30-199) over the stably
  sorted entries, run by one thread (see ref_harness.cpp) -> per-sphere force;
* ``ref_rigid.npz`` -- updateSphereDataCUDA, computeForcesAndTorquesCUDA,
  advectParticlesCUDA (physics_update.cu:26-310);
* ``ref_sap_<case>.npz`` -- sweepAndPruneCUDA
  (src/engine/cuda/collisions/SAP/sap_detection.cu:385-440) over sphere AABBs
  whose lower x extents are stably sorted as uint32 float bits -> 16-entry
  rows per sorted position (cleared to -1 before the launch);
* ``ref_morton_<case>.npz`` -- computeSpaceFillingCurveCUDA
  (sandbox/testLBVH.cu:113-151): boxes and a domain -> 30-bit Morton codes;
* ``ref_gjk.npz`` -- STARDUST::gjkCUDA (sandbox/testGJK.cu:237-315): convex
  point sets (world vertices) placed clearly apart or clearly overlapping
  by construction -> the kernel's verdict per pair (it prints a line for a
  hit and stores nothing, so each pair runs in its own launch and the
  printed lines are counted).

Usage:  python tests/golden/make_ref_golden.py OUT_DIR [hash rigid sap morton gjk]
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def harness():
    from oracle import ref_build
    lib_path = ref_build.build_harness()
    if lib_path is None:
        raise SystemExit("cannot build the harness")
    lib = C.CDLL(str(lib_path))
    lib.ref_last_error.restype = C.c_char_p
    return lib


def check(lib, rc, what):
    if rc != 0:
        raise SystemExit(f"{what}: {lib.ref_last_error().decode()}")


def dev(a):
    import torch
    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(np.uint8)).to("cuda").view(torch.uint8)


def ptr(t):
    return C.c_uint64(t.data_ptr())


def host(t, dtype, shape):
    return t.cpu().numpy().view(dtype).reshape(shape)


def hash_cases():
    rng = np.random.default_rng(2024)
    cases = {}
    n = 4096
    p = np.zeros((n, 4), np.float32)
    p[:, :3] = rng.uniform(0, 1, (n, 3))
    cases["a"] = (p, rng.uniform(0.002, 0.04, n).astype(np.float32), np.float32(1 / 32))
    n = 2048
    p = np.zeros((n, 4), np.float32)
    p[:, :3] = rng.uniform(0, 1, (n, 3))
    cases["b"] = (p, rng.uniform(0.01, 0.2, n).astype(np.float32), np.float32(0.4))
    cell = np.float32(1 / 8)
    vals = np.array([0.0, -0.0, -0.01, cell, 2 * cell, 0.0625, 0.1249999, 0.999, 1 - 1e-7, 1.0, 1.5],
                    np.float32)
    g = np.stack(np.meshgrid(vals, vals, vals, indexing="ij"), -1).reshape(-1, 3)
    p = np.zeros((len(g), 4), np.float32)
    p[:, :3] = g
    cases["c"] = (p, rng.uniform(0.0, 0.2, len(g)).astype(np.float32), cell)
    return cases


def run_hash(lib, out: Path):
    import torch
    results = {}
    for name, (pos, sizes, cell) in hash_cases().items():
        n = len(pos)
        cells = torch.zeros(9 * n, dtype=torch.int32, device="cuda")
        spheres = torch.zeros(9 * n, dtype=torch.int32, device="cuda")
        temp = torch.zeros(4, dtype=torch.int32, device="cuda")
        tpos, tsz = dev(pos), dev(sizes)
        check(lib, lib.ref_construct(C.c_uint(n), C.c_float(cell), ptr(cells), ptr(spheres), ptr(tsz), ptr(tpos),
                                     ptr(temp), C.c_uint(128), C.c_void_p(0)), "construct")
        res = dict(pos4=pos, sizes=sizes, cell_dim=np.float32(cell),
                   cells=host(cells, np.uint32, (-1,)), spheres=host(spheres, np.uint32, (-1,)),
                   count=np.uint32(host(temp, np.uint32, (-1,))[0]))
        np.savez_compressed(out / f"ref_hash_{name}.npz", **res)
        results[name] = res
        print(f"hash {name}: n={n} count={int(res['count'])}")
    return results


def run_traverse(lib, out: Path, hashed):
    import torch
    rng = np.random.default_rng(7)
    for name in ("a", "b"):
        h = hashed[name]
        n = len(h["pos4"])
        count = int(h["count"])
        order = np.argsort(h["cells"], kind="stable")
        ck, cv = h["cells"][order], h["spheres"][order]
        m = 16 * count + 2
        cells = np.full(m, 0xFFFFFFFF, np.uint32)
        sph = np.zeros(m, np.uint32)
        cells[:count], sph[:count] = ck[:count], cv[:count]
        vel = np.zeros((n, 4), np.float32)
        vel[:, :3] = rng.uniform(-1, 1, (n, 3))
        body = np.arange(n, dtype=np.int32) if name == "a" else (np.arange(n) // 4).astype(np.int32)
        force = torch.zeros(n * 4, dtype=torch.float32, device="cuda")
        temp = torch.tensor([16 * count, 0, 0, 0], dtype=torch.int32, device="cuda")
        mass = np.ones(n, np.float32)
        args = [dev(cells), dev(sph), dev(h["pos4"]), dev(vel), force, dev(mass), dev(h["sizes"]), dev(body)]
        check(lib, lib.ref_traverse_serial(*[ptr(a) for a in args], C.c_uint(n), ptr(temp), C.c_void_p(0)),
              "traverse")
        np.savez_compressed(out / f"ref_traverse_{name}.npz", cells=ck, spheres=cv, count=np.uint32(count),
                            pos4=h["pos4"], vel4=vel, body_of=body, force4=host(force, np.float32, (n, 4)))
        print(f"traverse {name}: entries={count}")


def rand_quat(rng, k):
    q = rng.normal(size=(k, 4)).astype(np.float32)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(np.float32)


def run_rigid(lib, out: Path):
    import torch
    rng = np.random.default_rng(11)
    nb = 300
    length = rng.integers(1, 8, nb).astype(np.int32)
    start = np.concatenate([[0], np.cumsum(length)[:-1]]).astype(np.int32)
    ns = int(length.sum())
    body_of = np.repeat(np.arange(nb, dtype=np.int32), length)
    f4 = lambda k, s=1.0: np.concatenate([rng.uniform(-s, s, (k, 3)), np.zeros((k, 1))], 1).astype(np.float32)
    init_rel, bpos, bvel, bomega = f4(ns, 0.05), f4(nb), f4(nb), f4(nb, 5.0)
    bquat = rand_quat(rng, nb)
    tens = [dev(x) for x in (init_rel, body_of, bpos, bvel, bquat, bomega)]
    pos = torch.zeros(ns * 4, dtype=torch.float32, device="cuda")
    rel = torch.zeros_like(pos)
    vel = torch.zeros_like(pos)
    check(lib, lib.ref_update_spheres(C.c_int(ns), C.c_int(nb), ptr(pos), ptr(vel), ptr(tens[0]), ptr(rel),
                                      ptr(tens[1]), ptr(tens[2]), ptr(tens[3]), ptr(tens[4]), ptr(tens[5]),
                                      C.c_void_p(0)), "update")
    upd = dict(u_pos=host(pos, np.float32, (ns, 4)), u_rel=host(rel, np.float32, (ns, 4)),
               u_vel=host(vel, np.float32, (ns, 4)))

    sforce = f4(ns, 2.0)
    bmass = rng.uniform(0.5, 20.0, nb).astype(np.float32)
    relin = f4(ns, 0.05)
    bf = torch.zeros(nb * 4, dtype=torch.float32, device="cuda")
    bt = torch.zeros_like(bf)
    t2 = [dev(x) for x in (bmass, start, length, relin, sforce, body_of)]
    check(lib, lib.ref_body_forces(C.c_int(ns), C.c_int(nb), ptr(bf), ptr(bt), *[ptr(t) for t in t2],
                                   C.c_void_p(0)), "body forces")
    frc = dict(f_force=host(bf, np.float32, (nb, 4)), f_torque=host(bt, np.float32, (nb, 4)))

    amass = rng.uniform(0.5, 5.0, nb).astype(np.float32)
    inertia = np.zeros((nb, 9), np.float32)
    for b in range(nb):
        qr = rand_quat(rng, 1)[0]
        s, x, y, z = qr
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - s * z), 2 * (x * z + s * y)],
                      [2 * (x * y + s * z), 1 - 2 * (x * x + z * z), 2 * (y * z - s * x)],
                      [2 * (x * z - s * y), 2 * (y * z + s * x), 1 - 2 * (x * x + y * y)]])
        d = rng.uniform(0.05, 2.0, 3) if b % 5 else rng.uniform(1e-3, 2e-2, 3)  # every fifth: det < 1e-4
        inertia[b] = (R @ np.diag(d) @ R.T).astype(np.float32).reshape(-1, order="F")
    a_in = dict(a_mass=amass, a_inertia=inertia, a_force=f4(nb, 3.0), a_torque=f4(nb, 0.5), a_pos=f4(nb),
                a_vel=f4(nb), a_omega=f4(nb), a_quat=rand_quat(rng, nb), a_lin=f4(nb, 2.0), a_ang=f4(nb, 0.3))
    d = {k: dev(v) for k, v in a_in.items()}
    check(lib, lib.ref_advect(C.c_int(ns), C.c_int(nb), C.c_float(1e-3), ptr(d["a_pos"]), ptr(d["a_vel"]),
                              ptr(d["a_omega"]), ptr(d["a_force"]), ptr(d["a_torque"]), ptr(d["a_quat"]),
                              ptr(d["a_mass"]), ptr(d["a_lin"]), ptr(d["a_ang"]), ptr(d["a_inertia"]),
                              C.c_void_p(0)), "advect")
    adv = {f"{k}_out": host(d[k], np.float32, a_in[k].shape) for k in ("a_pos", "a_vel", "a_omega", "a_quat",
                                                                      "a_lin", "a_ang")}
    np.savez_compressed(out / "ref_rigid.npz", init_rel=init_rel, body_of=body_of, bpos=bpos, bvel=bvel,
                        bquat=bquat, bomega=bomega, start=start, length=length, sforce=sforce, bmass=bmass,
                        relin=relin, **upd, **frc, **a_in, **adv)
    print(f"rigid: {nb} bodies, {ns} spheres")


def run_sap(lib, out: Path):
    import torch
    from oracle import oracle as orc
    for name, n, rlo, rhi, seed in (("a", 3000, 0.002, 0.01, 21), ("b", 2000, 0.01, 0.04, 22)):
        rng = np.random.default_rng(seed)
        pos = np.zeros((n, 4), np.float32)
        pos[:, :3] = rng.uniform(0.05, 0.95, (n, 3))
        pos[:, 3] = rng.uniform(rlo, rhi, n)
        r = pos[:, 3]
        upperx = (pos[:, 0] + r).astype(np.float32)
        uppery = (pos[:, 1] + r).astype(np.float32)
        lowery = (pos[:, 1] - r).astype(np.float32)
        keys = (pos[:, 0] - r).astype(np.float32).view(np.uint32).copy()
        ids = np.arange(n, dtype=np.uint32)
        ks, vs = orc.radix_sort_pairs(keys, ids, 32)
        lowerx_sorted = ks.view(np.float32)
        rows = dev(np.full((n, 16), -1, np.int32))
        d = [dev(a) for a in (upperx, lowerx_sorted, uppery, lowery, vs, ids)]
        torch.cuda.synchronize()
        check(lib, lib.ref_sap_sweep(n, *[ptr(t) for t in d], ptr(rows), C.c_void_p(0)), "sap sweep")
        torch.cuda.synchronize()
        res = host(rows, np.int32, (n, 16))
        np.savez_compressed(out / f"ref_sap_{name}.npz", pos=pos, upperx=upperx, lowerx_sorted=lowerx_sorted,
                            uppery=uppery, lowery=lowery, idx_sorted=vs, rows=res)
        print(f"sap {name}: {n} boxes, {(res >= 0).sum()} row entries")


def run_morton(lib, out: Path):
    for name, n, seed, span in (("a", 5000, 31, 1.0), ("b", 3000, 32, 0.25)):
        rng = np.random.default_rng(seed)
        # a domain around the origin; some box centres outside it (clamped
        # codes) and on both sides of its centre (the floor of negatives)
        glo = np.array([-1.0, -0.5, -2.0, 0.0], np.float32) * span
        ghi = np.array([1.5, 0.75, 1.0, 0.0], np.float32) * span
        c = rng.uniform(glo[:3] - 0.1 * span, ghi[:3] + 0.1 * span, (n, 3)).astype(np.float32)
        h = rng.uniform(0.0, 0.01 * span, (n, 3)).astype(np.float32)
        L = np.zeros((n, 4), np.float32)
        H = np.zeros((n, 4), np.float32)
        L[:, :3] = c - h
        H[:, :3] = c + h
        if name == "b":  # the domain as the LBVH builds it: the boxes' bounds (testLBVH.cu:61-77)
            glo = np.concatenate([L[:, :3].min(0), [0.0]]).astype(np.float32)
            ghi = np.concatenate([H[:, :3].max(0), [0.0]]).astype(np.float32)
        rows = np.concatenate([H, L], 1)  # the sandbox AABB: upper extent, then lower extent
        d_rows, d_codes, d_idx = dev(rows), dev(np.zeros(n, np.uint32)), dev(np.zeros(n, np.int32))
        import torch
        torch.cuda.synchronize()
        check(lib, lib.ref_morton(n, ghi.ctypes.data_as(C.c_void_p), glo.ctypes.data_as(C.c_void_p), ptr(d_rows),
                                  ptr(d_codes), ptr(d_idx), C.c_void_p(0)), "morton")
        codes = host(d_codes, np.uint32, (n,))
        np.savez_compressed(out / f"ref_morton_{name}.npz", lo=L, hi=H, glo=glo, ghi=ghi, codes=codes)
        print(f"morton {name}: {n} boxes, {len(np.unique(codes))} distinct codes")


HULL_DTYPE = np.dtype({"names": ["type", "group_owner", "is_active", "is_visible", "vertex_idx", "n_vertices",
                                 "mass", "radius", "position", "force", "torque"],
                       "formats": ["<u4", "<u4", "u1", "u1", "<i4", "<i4", "<f4", "<f4", ("<f4", 4), ("<f4", 4),
                                   ("<f4", 4)],
                       "offsets": [0, 4, 8, 9, 12, 16, 20, 24, 32, 48, 64], "itemsize": 80})  # primitives.hpp


def gjk_cases(n_pairs: int, seed: int):
    """Pairs of convex point sets (8-32 points on a jittered sphere around
    their centre), placed along a random direction u either apart by a gap
    beyond their support extents along u (separated by construction) or
    closer than the sum of their inscribed-ball radii (overlapping by
    construction); gaps and overlaps of 30 %, 5 % and 1 % of the size."""
    from scipy.spatial import ConvexHull
    rng = np.random.default_rng(seed)

    def shape():
        while True:
            k = int(rng.integers(8, 33))
            d = rng.normal(size=(k, 3))
            pts = d / np.linalg.norm(d, axis=1, keepdims=True) * rng.uniform(0.85, 1.0, (k, 1))
            pts *= rng.uniform(0.5, 1.5)
            rin = float(np.min(-ConvexHull(pts).equations[:, 3]))
            if rin > 0.1 * np.abs(pts).max():
                return pts, rin

    cen, pts_all, pairs, truth = [], [], [], []
    for i in range(n_pairs):
        (pa, ra), (pb, rb) = shape(), shape()
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        ca = rng.uniform(-5.0, 5.0, 3)
        frac = (0.3, 0.05, 0.01)[(i // 2) % 3]
        if i % 2 == 0:
            gap = frac * min(np.abs(pa).max(), np.abs(pb).max())
            cb = ca + u * ((pa @ u).max() + (pb @ -u).max() + gap)
        else:
            cb = ca + u * (ra + rb - frac * min(ra, rb))
        for c, p in ((ca, pa), (cb, pb)):
            cen.append(c)
            pts_all.append(p)
        pairs.append((2 * i, 2 * i + 1))
        truth.append(i % 2 == 1)
    return cen, pts_all, np.array(pairs, np.int32), np.array(truth)


class StdoutCapture:
    """Collects what the process writes to file descriptor 1 (device printf
    output is written there at synchronisation)."""

    def __enter__(self):
        import os
        import tempfile
        self.libc = C.CDLL(None)
        self.libc.fflush(None)
        sys.stdout.flush()
        self.saved = os.dup(1)
        self.tmp = tempfile.TemporaryFile()
        os.dup2(self.tmp.fileno(), 1)
        return self

    def __exit__(self, *exc):
        import os
        self.libc.fflush(None)
        os.dup2(self.saved, 1)
        os.close(self.saved)
        self.tmp.seek(0)
        self.text = self.tmp.read().decode(errors="replace")
        self.tmp.close()


def run_gjk(lib, out: Path):
    import torch
    cen, pts, pairs, truth = gjk_cases(600, 41)
    counts = np.array([len(p) for p in pts], np.int32)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int32)
    verts = np.zeros((counts.sum(), 4), np.float32)
    hulls = np.zeros(len(pts), HULL_DTYPE)
    for k, (c, p) in enumerate(zip(cen, pts)):
        w = (np.asarray(c)[None, :] + p).astype(np.float32)
        verts[starts[k]:starts[k] + counts[k], :3] = w
        hulls[k]["type"] = 2  # POLYHEDRA
        hulls[k]["is_active"] = 1
        hulls[k]["vertex_idx"] = starts[k]
        hulls[k]["n_vertices"] = counts[k]
        hulls[k]["mass"] = 1.0
        hulls[k]["radius"] = -1.0
        hulls[k]["position"][:3] = np.asarray(c, np.float32)
    d_h, d_v = dev(hulls.view(np.uint8)), dev(verts)
    verdict = np.zeros(len(pairs), bool)
    for i, (a, b) in enumerate(pairs):
        d_p = dev(np.array([a, b, -1, -1], np.int32))
        torch.cuda.synchronize()
        with StdoutCapture() as cap:
            check(lib, lib.ref_gjk_one(len(pts), ptr(d_p), ptr(d_h), ptr(d_v), C.c_void_p(0)), "gjk")
        verdict[i] = "collided" in cap.text
    np.savez_compressed(out / f"ref_gjk.npz", verts=verts, starts=starts, counts=counts,
                        centres=np.asarray(cen, np.float32), pairs=pairs, truth=truth, verdict=verdict)
    print(f"gjk: {len(pairs)} pairs, reference verdicts agree with the construction on "
          f"{int((verdict == truth).sum())} (separated {int((~verdict & ~truth).sum())}/{int((~truth).sum())}, "
          f"overlapping {int((verdict & truth).sum())}/{int(truth.sum())})")


def main():
    out = Path(sys.argv[1] if len(sys.argv) > 1 else ".")
    out.mkdir(parents=True, exist_ok=True)
    import torch
    torch.cuda.init()
    torch.zeros(1, device="cuda")  # make the primary context current
    lib = harness()
    check(lib, lib.ref_init(str(ROOT / "oracle" / "_ref").encode()), "init")
    parts = sys.argv[2:] or ["hash", "rigid", "sap", "morton", "gjk"]
    if "hash" in parts:
        hashed = run_hash(lib, out)
        run_traverse(lib, out, hashed)
    if "rigid" in parts:
        run_rigid(lib, out)
    if "sap" in parts:
        run_sap(lib, out)
    if "morton" in parts:
        run_morton(lib, out)
    if "gjk" in parts:
        run_gjk(lib, out)


if __name__ == "__main__":
    main()
