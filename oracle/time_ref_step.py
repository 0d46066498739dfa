"""Times the reference's own GPU step on the 1,048,576-sphere settling box.

Test/measurement infrastructure (not the product): runs the reference's
spatial-hash step -- its own kernels, compiled unchanged from its sources by
oracle/ref_build.py, launched by oracle/ref_harness.cpp with the reference's
launch shapes (ref_step_async) -- on the same scene bench.py uses, and prints
one JSON line with ms per step and sphere-steps/s.

The reference hashes in [0, 1)^3 with 8 bits per axis, so the 1 x 1 x 2 m box
is mapped by x' = x / 2 (cell 0.02 -> 0.01, 100 cells per axis) and sizes are
diameters of the mapped spheres, as the reference engine stores them.

Only the stages are timed, each on the packed scene as generated: the key
construction, the reference's sort as written (its output is not a
permutation -- sh_collision_detection.cu:241-242 -- but it does a correct
sort's work), the traversal fed a correctly sorted list, and the rigid-body
update (last: it moves the spheres).  The step as written is not run: its
traversal reads its input from that broken sort and races on its entry
counter (collision_resolution.cu:117-120), and a bench run whose last
phases were this leg (then timing that step, repeated on its own evolving
state) and a 15-second CPU baseline did not end within its 45-minute limit
(the GPU still answered).  Timing: CUDA events on the launch stream around
each stage, the L2 flushed (256 MB write) before each; `warmup` untimed
key constructions first.

Usage: python oracle/time_ref_step.py [--steps K] [--warmup W] [--n N]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


class RefStep(C.Structure):
    _fields_ = [("n", C.c_uint), ("cell_dim", C.c_float)] + [
        (k, C.c_uint64) for k in (
            "cells", "spheres", "cells_tmp", "spheres_tmp", "radices", "radix_sums", "d_temp", "pos", "vel",
            "force", "size", "mass", "rigid", "init_rel", "rel", "bpos", "bvel", "bomega", "bforce", "btorque",
            "bquat", "bmass", "lin", "ang", "inertia", "start", "length")] + [("dt", C.c_float)]


def measure(steps: int = 10, warmup: int = 3, n: int = 1 << 20, scene=None) -> dict:
    """Times the reference's GPU step (see the module docstring); returns the
    JSON-able result, or {"unavailable": why} when its kernels are not built.
    scene: (pos4, vel4, dt) of the settling box when already generated."""
    import types
    args = types.SimpleNamespace(steps=steps, warmup=warmup, n=n)
    import torch
    from oracle import ref_build
    from stardust_gb300 import scenes

    cub = ROOT / "oracle" / "_ref"
    if not all((cub / f"{s}.cubin").exists() for s in ref_build.SOURCES):
        return {"impl": "reference-gpu", "unavailable": "reference kernels not built (oracle/ref_build.py)"}
    lib_path = ref_build.build_harness()
    if lib_path is None:
        return {"impl": "reference-gpu", "unavailable": "the launch harness did not compile"}
    lib = C.CDLL(str(lib_path))
    lib.ref_last_error.restype = C.c_char_p
    torch.zeros(1, device="cuda")
    if lib.ref_init(str(cub).encode()) != 0:
        return {"impl": "reference-gpu", "unavailable": lib.ref_last_error().decode()}

    n = args.n
    if scene is not None:
        pos, vel, dt = scene
        n = len(pos)
    else:
        box = (1.0, 1.0, 2.0) if n == 1 << 20 else scenes.scaled_box(n)
        t0 = time.time()
        pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=box, seed=0)
        print(f"scene: {n} spheres in {time.time() - t0:.1f}s", file=sys.stderr)
    dev = torch.device("cuda")
    f4 = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)
    p = pos.copy()
    p[:, :3] *= 0.5
    p[:, 3] = 0.0
    v = vel.copy()
    v[:, :3] *= 0.5
    v[:, 3] = 0.0
    size = (pos[:, 3]).astype(np.float32)  # diameter of the halved sphere
    mass = vel[:, 3].astype(np.float32)
    keep = {}

    def buf(name, t):
        keep[name] = t
        return t.data_ptr()

    u32 = lambda k: torch.zeros(k, dtype=torch.int32, device=dev)
    s = RefStep()
    s.n, s.cell_dim, s.dt = n, 0.01, dt
    s.cells, s.spheres, s.cells_tmp, s.spheres_tmp = (buf(k, u32(9 * n)) for k in ("c", "s", "ct", "st"))
    s.radices, s.radix_sums, s.d_temp = buf("r", u32(16 * 256 * 12)), buf("rs", u32(256)), buf("t", u32(4))
    s.pos, s.vel, s.force = buf("p", f4(p)), buf("v", f4(v)), buf("f", f4(np.zeros_like(p)))
    s.size, s.mass = buf("sz", f4(size)), buf("m", f4(mass))
    s.rigid = buf("rg", torch.arange(n, dtype=torch.int32, device=dev))
    s.init_rel, s.rel = buf("ir", f4(np.zeros_like(p))), buf("rl", f4(np.zeros_like(p)))
    s.bpos, s.bvel = buf("bp", f4(p)), buf("bv", f4(v))
    s.bomega, s.bforce, s.btorque = (buf(k, f4(np.zeros_like(p))) for k in ("bw", "bf", "bt"))
    q = np.zeros_like(p)
    q[:, 0] = 1.0
    s.bquat, s.bmass = buf("bq", f4(q)), buf("bm", f4(mass))
    lin = np.zeros_like(p)
    lin[:, :3] = v[:, :3] * mass[:, None]
    s.lin, s.ang = buf("li", f4(lin)), buf("an", f4(np.zeros_like(p)))
    s.inertia = buf("in", torch.zeros(9 * n, dtype=torch.float32, device=dev))
    s.start = buf("s0", torch.arange(n, dtype=torch.int32, device=dev))
    s.length = buf("ln", torch.ones(n, dtype=torch.int32, device=dev))

    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def run(stages):
        if lib.ref_stages_async(C.byref(s), stages, sp) != 0:
            raise SystemExit(lib.ref_last_error().decode())

    def timed(stages, before=None):
        out = []
        for k in range(args.steps):
            if before:
                before()
            flush.fill_(k & 0xFF)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            run(stages)
            b.record(stream)
            b.synchronize()
            out.append(a.elapsed_time(b))
        return out

    for _ in range(args.warmup):
        run(1)
    torch.cuda.synchronize()
    # stages alone, on the packed scene; the traversal is fed a correctly
    # (stably) sorted list made by this library's onesweep sort, so its cost
    # is the intended one
    from stardust_gb300 import SpatialPartition
    sort_scratch = torch.zeros((SpatialPartition.sort_scratch_bytes(9 * n, 32) + 3) // 4, dtype=torch.int32,
                               device=dev)

    def construct_and_sort_correctly():
        run(1)
        SpatialPartition.sort_collision_list(keep["c"], keep["s"], keep["ct"], keep["st"], 9 * n, sort_scratch)

    st_construct = timed(1)
    st_sort = timed(2, before=lambda: run(1))
    st_traverse = timed(4, before=construct_and_sort_correctly)
    st_rigid = timed(8)
    med = lambda x: sorted(x)[len(x) // 2]
    staged = med(st_construct) + med(st_sort) + med(st_traverse) + med(st_rigid)
    return {
        "impl": "reference-gpu", "metric": "particle-steps/s @1M spheres", "n_spheres": n, "steps": args.steps,
        "ms_per_step": staged, "value": n / (staged * 1e-3), "unit": "particle-steps/s",
        "ms_stages_median": {"construct": med(st_construct), "sort_as_written": med(st_sort),
                             "traverse_sorted_input": med(st_traverse), "rigid_body": med(st_rigid)},
        "as_written_step": "not run: its traversal reads the broken sort's output and races on its entry "
                           "counter; a run that timed it on its own evolving state did not end",
        "kernels": "constructCollisionList + 4x(Tabulate, Sum, Reorder) over 9n entries + "
                   "tranverseCollisionList + computeForcesAndTorques + advect + updateSphereData"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--n", type=int, default=1 << 20)
    args = ap.parse_args()
    print(json.dumps(measure(args.steps, args.warmup, args.n)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
