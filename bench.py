"""Benchmark of the DEM step: particle-steps/s at 1,048,576 polydisperse spheres.

Workload: the settling box -- 1,048,576 spheres, radii lognormal (median
5 mm, sigma 0.25) clipped to [2.5, 10] mm, random sequential addition in a
walled 1 x 1 x 2 m box, linear spring-dashpot kn = 1e5, restitution 0.5,
Coulomb mu = 0.3, gravity, dt = 5e-6 s, hash cell 2 x max radius (50 x 50 x
100 cells), cell keys sorted every step, a 2,000-step run.  Synthetic,
seeded.

One step = contact gather + integration (over contact lists with a skin
between list builds), a stable sort of the (cell key, slot) pairs -- an
incremental re-sort of the keys that changed, or the onesweep radix passes
--, reorder + cell_start.  The scene is first advanced (untimed) to step
`--advance` (1,000) of the run, so the timed window sits in the middle of
the settling run rather than right after the packing.  Timings:

  value      device time per step (CUDA events on the engine's stream, one
             event pair per step, the L2 flushed by a 256 MB write before
             every timed step), whole job over ranks; also the first steps
             after the packing (early_window), the same state without
             contact lists and with the full radix sort every step;
  e2e        the same steps through the public C ABI with the state in
             pinned host memory: per step, upload positions + velocities
             (sd_engine_set_state), step, read positions + velocities back
             into the same buffers (sd_engine_get_state);
  roofline   the dominant kernel (contact + integrate) timed alone on the
             same stream, its algorithmic bytes / duration against the
             measured HBM peak;
  cpu_baseline  the CPU oracle (the restated step, OpenMP on the host cores)
             on a bounded sample of the same scene;
  dense_bed  the same spheres with radii x1.2 (~2.5M contact pairs), after
             1,000 steps;
  reference_gpu  with --ref-gpu only: the reference's own GPU kernels
             (compiled unchanged from its sources, oracle/time_ref_step.py)
             timed stage by stage on the same scene and GPU, beside this
             step's time (a baseline leg);
  drum       the rotating drum: 2.1M spheres and clumps against a turning
             20,480-triangle cylinder (bench_drum);
  batch      512 independent scenes (~2.9M spheres) stepped together, one
             launch per stage (bench_batch), against 16 of them stepped alone;
  sap        the sweep-and-prune operators on 2,000,000 boxes, beside the
             reference's recorded SAP run times (bench_sap);
  gjk        the second half of the metric: mean GJK support evaluations per
             candidate pair with the learned warm start vs plain GJK, on a
             65,536-hull scene (bench_hulls), with the contact sets and states
             of the two runs compared.

``--impl reference`` times the reference path on the host cores.  The
reference has no CPU DEM path (its Device::CPU is never read), so this arm
runs the CPU restatement of the step (oracle/) with all host threads.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "particle-steps/s @1M spheres"
UNIT = "particle-steps/s"
N_FULL = 1 << 20
# algorithmic HBM bytes per sphere of one launch of the contact+integrate
# kernel: read own position/velocity/spin (48), write next position/velocity/
# spin (48) + cell key + slot (8); the cell_start table (250,001 words for
# 1,048,576 spheres) adds ~1 B/sphere
CONTACT_BYTES_PER_SPHERE = 48 + 48 + 8
# with contact lists (knob skin_um), a listed step also reads the sphere's
# list count (4) and its position at the last build (16) for the skin check;
# the listed neighbours' ids and slots add 8 B per entry (not counted: a
# sphere of the settling box lists ~1-2 neighbours)
LIST_BYTES_PER_SPHERE = 4 + 16
# algorithmic HBM bytes per sphere-step of the whole step (2 sort passes of
# 18-bit keys):  contact 104 + histogram 4 + 2 x (8 read + 8 write) + reorder
# (slot 4 + key 4 + gather 48 + write 48)
STEP_BYTES_PER_SPHERE = 104 + 4 + 32 + 104


def clocks_mhz(clocks) -> float:
    """Median SM clock seen during the timed region (max clock if unsampled)."""
    try:
        v = float(clocks.get("sm_mhz") or 0)
    except Exception:
        v = 0.0
    return v if v > 0 else 2070.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def build_scene(n: int, seed: int, rsa=None):
    from stardust_gb300 import scenes
    box = (1.0, 1.0, 2.0) if n == N_FULL else scenes.scaled_box(n)
    t0 = time.time()
    pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=box, seed=seed, rsa=rsa)
    log(f"scene: {n} spheres, volume fraction {phi:.4f}, generated in {time.time() - t0:.1f}s")
    return pos, vel, cfg, dt, phi


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = None

    def __enter__(self):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            d = json.loads(f.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def recorded_profile(kind: str = "scan"):
    """DRAM bytes and warp instructions per sphere of one contact-kernel
    launch, from the committed ncu summary (profiles/roofline_traffic.json):
    kind "scan" (the candidate scan) or "listed" (contact lists)."""
    f = ROOT / "profiles" / "roofline_traffic.json"
    if f.exists():
        try:
            d = json.loads(f.read_text())
            pre = "contact_integrate" if kind == "scan" else "contact_listed"
            return d.get(f"{pre}_bytes_per_sphere"), d.get(f"{pre}_warp_instructions_per_sphere")
        except Exception:
            pass
    return None, None


SMS, SCHEDULERS_PER_SM = 152, 4  # GB300: one warp instruction per scheduler per clock


def cpu_oracle_rate(pos, vel, cfg, dt, seconds: float, threads: int | None, z_div: int | None = None):
    """Oracle steps on the host cores until ~`seconds` of work: particle-steps/s."""
    from oracle import oracle as orc
    p = orc.derive_params(cfg, pos[:, 3], dt, z_div)
    if threads:
        orc.lib().sdo_set_num_threads(threads)
    used = orc.lib().sdo_num_threads()
    n = len(pos)
    omg = orc.with_ids(np.zeros_like(pos), np.arange(n))
    sp, sv, sw, _, cs = orc.prepare(p, pos, vel, omg)
    steps = 0
    t0 = time.perf_counter()
    while True:
        pn, vn, wn, keys, _, _, _ = orc.contact_integrate(p, sp, sv, sw, cs, record=False)
        sp, sv, sw, _, cs = orc.sort_reorder(p, pn, vn, wn, keys)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return n * steps / el, used, steps, el


def run_reference_arm(args, rank, world):
    """The CPU restatement of the step on all host threads, on the same
    scene; the scene comes from the oracle's copy of the seeded builders and
    the parameters from the oracle's own derivation, so this arm loads
    nothing of the library."""
    if rank != 0:
        return 0
    n = args.n
    from oracle import oracle as orc
    pos, vel, cfg, dt, phi = build_scene(n, args.seed, rsa=orc.scene_rsa)
    p = orc.derive_params(cfg, pos[:, 3], dt, args.z_div)
    used = orc.lib().sdo_num_threads()
    omg = orc.with_ids(np.zeros_like(pos), np.arange(n))
    # the same window of the settling run as the GPU arm: advanced untimed
    # (sdo_run) to step `advance`, then warm-up and the timed steps
    sp, sv, sw = orc.run(p, pos, vel, omg, args.advance)
    sp, sv, sw, _, cs = orc.prepare(p, sp, sv, sw)
    for _ in range(args.warmup):
        pn, vn, wn, keys, _, _, _ = orc.contact_integrate(p, sp, sv, sw, cs, record=False)
        sp, sv, sw, _, cs = orc.sort_reorder(p, pn, vn, wn, keys)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pn, vn, wn, keys, _, _, _ = orc.contact_integrate(p, sp, sv, sw, cs, record=False)
        sp, sv, sw, _, cs = orc.sort_reorder(p, pn, vn, wn, keys)
    el = time.perf_counter() - t0
    v = n * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"settling box, {n} polydisperse spheres, 1x1x2 m, dt 5e-6 s, 2000-step run",
                   "n_spheres": n, "volume_fraction": round(phi, 4), "l2": "n/a (host cores)",
                   "timed_window": f"steps {args.advance + args.warmup + 1}-{args.advance + args.warmup + args.steps} "
                                   "of the run"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": used, "kind": "port",
                         "sample": f"{args.steps} full steps (after {args.advance + args.warmup}) of the {n}-sphere "
                                   "scene, CPU restatement of the step (the reference has no CPU DEM path), OpenMP "
                                   "on all host threads"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


ONLINE_EVERY, ONLINE_ITERS, ONLINE_LR = 5, 10, 2e-3


def bench_hulls(n_hulls: int, steps: int, warmup: int, local: int):
    """GJK support evaluations per candidate pair, plain vs learned seed, on
    the convex-hull step (65,536 hulls of 8-32 points, 0.02 m across, random
    orientations, packed at 1.95 radii in a walled 1 m box).  Four engines
    step the same scene: plain GJK; the previous step's direction as seed
    (the untrained residual network); the network trained offline on the
    separating directions plain GJK logged in 10 steps; the network trained
    online from scratch during the run (every ONLINE_EVERY steps, ONLINE_ITERS
    Adam steps on that step's max-margin targets, timed steps included).
    After `warmup` steps each, `steps` steps are timed with CUDA events."""
    import torch
    import stardust_gb300 as sd
    from stardust_gb300 import _abi, scenes
    pts, pos, quat, vel, mass, cfg, dt = scenes.hull_box(n_hulls, seed=3, box=(1.0, 1.0, 1.0), spacing=0.0195,
                                                          vmax=0.3)
    cfg.cuda_device = local

    def engine(mode, params=None):
        e = sd.DEMEngine(cfg)
        sd.add_hull_scene(e, pts, pos, quat, vel, mass)
        e.prepare()
        if params is not None:
            e.set_mlp_params(params)
        e.set_gjk_seed(mode)
        return e

    rng = np.random.default_rng(0)
    plain = engine(_abi.SD_GJK_SEED_PLAIN)
    X, T = [], []
    for _ in range(10):
        plain.step(dt, 1)
        e = plain.hull_entries()
        selfs = np.repeat(np.arange(len(e["off"]) - 1), np.diff(e["off"]))
        m = np.flatnonzero((e["partners"] > selfs) & (e["status"] == 0) & (e["feat"][:, 7] == 1))
        m = m[rng.permutation(len(m))[:20000]]
        d = e["dir"][m, :3]
        X.append(e["feat"][m])
        T.append(np.concatenate([d / np.linalg.norm(d, axis=1, keepdims=True), np.ones((len(m), 1))], 1))
    Xt = torch.from_numpy(np.concatenate(X).astype(np.float32)).cuda()
    Tt = torch.from_numpy(np.concatenate(T).astype(np.float32)).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain.mlp_train(Xt, Tt, 400, 2e-3)
    train_s = time.perf_counter() - t0
    params = plain.mlp_params()
    plain.close()
    out = {"workload": f"{n_hulls} convex hulls (8-32 points, 0.02 m across), packed in a walled 1 m box, dt 1e-5 s",
           "train_samples": int(Xt.shape[0]), "train_iters": 400, "train_s": train_s,
           "online": {"every": ONLINE_EVERY, "iters": ONLINE_ITERS, "lr": ONLINE_LR, "warmup_steps": warmup}}
    engines = {k: engine(m, params) for k, m in (("plain", _abi.SD_GJK_SEED_PLAIN),
                                                   ("learned", _abi.SD_GJK_SEED_LEARNED),
                                                   ("previous", _abi.SD_GJK_SEED_PREVIOUS))}
    # the network trained online from scratch (untrained = the previous
    # direction), on max-margin targets of the run's own pairs; it keeps
    # training through the timed steps
    engines["online"] = engine(_abi.SD_GJK_SEED_LEARNED)
    engines["online"].set_gjk_training(ONLINE_EVERY, ONLINE_ITERS, ONLINE_LR)
    for k, e in engines.items():
        e.step(dt, warmup)
        e.sync()
        st = torch.cuda.ExternalStream(e.stream(), device=torch.device("cuda", local))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        iters = pairs = 0
        a.record(st)
        for _ in range(steps):
            e.step(dt, 1)
        b.record(st)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / steps
        for _ in range(3):  # counters of single steps
            e.step(dt, 1)
            s2 = e.stats()
            iters += s2["gjk_iters"]
            pairs += s2["gjk_pairs"]
        out[f"ms_per_step_{k}"] = ms
        out[f"iters_per_pair_{k}"] = iters / max(pairs, 1)
        out[f"contacts_{k}"] = s2["contacts"]
        out["pairs_per_step"] = s2["gjk_pairs"]
    hp = engines["plain"].hull_entries()
    hl = engines["learned"].hull_entries()
    out["identical_contacts"] = bool(np.array_equal(hp["status"] == 1, hl["status"] == 1))
    out["identical_state"] = bool(np.array_equal(engines["plain"].bodies(_abi.SD_BODY_POSITION).view(np.uint32),
                                                 engines["learned"].bodies(_abi.SD_BODY_POSITION).view(np.uint32)))
    ho = engines["online"].hull_entries()
    out["identical_contacts_online"] = bool(np.array_equal(hp["status"] == 1, ho["status"] == 1))
    out["ratio_plain_over_learned"] = out["iters_per_pair_plain"] / out["iters_per_pair_learned"]
    out["ratio_plain_over_online"] = out["iters_per_pair_plain"] / out["iters_per_pair_online"]
    out["ratio_previous_over_online"] = out["iters_per_pair_previous"] / out["iters_per_pair_online"]
    out["hull_steps_per_s_learned"] = n_hulls / (out["ms_per_step_learned"] * 1e-3)
    for k in ("plain", "learned"):
        out[f"narrow_roofline_{k}"] = narrow_roofline(engines[k], local)
    for e in engines.values():
        e.close()
    return out


# Compulsory HBM bytes of one unique hull pair in the narrow phase besides its
# vertices: the unique-list entry, its self and partner ids (12); per body
# position and quaternion (2 x 32) and its vertex range (2 x 8); the seed
# (16); written for the entry and its mirror: direction, force, torque, info
# (2 x 52).
NARROW_BYTES_PER_PAIR = 12 + 64 + 16 + 16 + 104


def narrow_roofline(eng, local: int, reps: int = 10):
    """The narrow phase (GJK, EPA on the hits, contact forces) launched alone
    on the last step's lists, timed with CUDA events after a 256 MB write;
    algorithmic bytes per unique pair = one read of both hulls' vertices
    (16 B each) + NARROW_BYTES_PER_PAIR.  Also the vertex bytes the support
    evaluations load (iterations x both hulls), the re-read factor."""
    import torch
    from stardust_gb300 import _abi
    ent = eng.hull_entries()
    _, vc, _ = eng.hull_shapes()
    selfs = np.repeat(np.arange(len(ent["off"]) - 1), np.diff(ent["off"]))
    u = ent["partners"] > selfs
    nv = vc[selfs[u]].astype(np.int64) + vc[ent["partners"][u]].astype(np.int64)
    pairs = int(u.sum())
    min_bytes = 16 * int(nv.sum()) + NARROW_BYTES_PER_PAIR * pairs
    loaded_vertex_bytes = 16 * int((nv * ent["iters"][u]).sum())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    st = torch.cuda.ExternalStream(eng.stream(), device=torch.device("cuda", local))
    a = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    b = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    for i in range(reps):
        with torch.cuda.stream(st):
            flush.fill_(i & 0xFF)
        a[i].record(st)
        _abi.call("sd_engine_launch_stage", eng._h, _abi.SD_STAGE_CONTACT, 0.0, h=eng._h)
        b[i].record(st)
    torch.cuda.synchronize()
    eng.sync()
    ms = sum(x.elapsed_time(y) for x, y in zip(a, b)) / reps
    peak, kind = measured_peak()
    achieved = min_bytes / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "unique_pairs": pairs, "hits": int((ent["status"][u] == 1).sum()),
            "bytes_per_pair": min_bytes / max(pairs, 1), "vertex_bytes_per_pair": 16 * float(nv.mean()) if pairs else 0,
            "loaded_vertex_bytes_per_pair": loaded_vertex_bytes / max(pairs, 1), "ms": ms,
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": kind,
            "pairs_per_s": pairs / (ms * 1e-3)}


def bench_batch(n_scenes: int, steps: int, warmup: int, local: int, tune: bool):
    """Batched scenes: n_scenes independent walled boxes (sphere counts
    lognormal in [256, 65,536], median 4,096; ~2.9M spheres for 512 scenes;
    r = 0.01 m at 35 % volume fraction, dt 1e-5 s) stepped together, one
    launch per stage, timed with CUDA events (the working set exceeds L2,
    and a 256 MB write still precedes every timed step).  For comparison, 16
    scenes spread over the size range are stepped alone, one engine each."""
    import torch
    import stardust_gb300 as sd
    from stardust_gb300 import scenes
    batch, cfg, dt = scenes.batch_boxes(n_scenes=n_scenes, seed=11)
    cfg.cuda_device = local
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def timed(eng, k):
        st = torch.cuda.ExternalStream(eng.stream(), device=torch.device("cuda", local))
        a = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
        b = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
        for i in range(k):
            with torch.cuda.stream(st):
                flush.fill_(i & 0xFF)
            a[i].record(st)
            eng.step(dt, 1)
            b[i].record(st)
        torch.cuda.synchronize()
        return sum(x.elapsed_time(y) for x, y in zip(a, b)) / k

    eng = sd.DEMEngine(cfg)
    for pos, vel, lo, hi in batch:
        eng.add_scene(pos, vel, lo, hi)
    eng.prepare()
    eng.step(dt, warmup)
    eng.sync()
    tuned = None
    if tune:
        from stardust_gb300 import autotune
        tuned = autotune.tune_engine(eng, dt, reps=3)
    ms = timed(eng, steps)
    st = eng.stats()
    eng.close()
    counts = np.array([len(b[0]) for b in batch])
    total = int(counts.sum())
    order = np.argsort(counts)
    pick = order[np.linspace(0, len(order) - 1, 16).astype(int)]
    alone_ms, alone_n = 0.0, 0
    for k in pick:
        pos, vel, lo, hi = batch[k]
        e1 = sd.DEMEngine(cfg)
        e1.add_scene(pos, vel, lo, hi)
        e1.prepare()
        e1.step(dt, warmup)
        e1.sync()
        alone_ms += timed(e1, max(steps // 2, 3))
        alone_n += len(pos)
        e1.close()
    return {"workload": f"{n_scenes} independent walled boxes, {total} spheres (r 0.01 m, 35 % volume fraction), "
                        f"counts lognormal in [256, 65536], median 4096, dt 1e-5 s",
            "scenes": n_scenes, "spheres": total, "cells": st["n_cells"],
            "count_quantiles": [int(np.quantile(counts, q)) for q in (0.0, 0.25, 0.5, 0.75, 1.0)],
            "ms_per_step": ms, "particle_steps_per_s": total / (ms * 1e-3),
            "per_scene_particle_steps_per_s_median": float(np.median(counts)) / (ms * 1e-3),
            "alone_16_scenes": {"spheres": alone_n, "ms_per_step_sum": alone_ms,
                                "particle_steps_per_s": alone_n / (alone_ms * 1e-3)},
            "device_errors": st["device_errors"], "moved_keys_last_step": st["moved_keys"], "autotune": tuned}


def bench_drum(steps: int, warmup: int, local: int, tune: bool = True):
    """The rotating drum (drum_scene): 2,097,152 spheres -- 10 % of the bodies
    4-sphere clumps -- in a closed cylinder of radius 0.5 m and length 0.5 m
    meshed with 20,480 triangles, turning at 2 rad/s, dt 2e-6 s; radii
    U[1.2, 2.4] mm (the specified U[2, 4] mm would fill 67 % of the drum's
    volume, beyond random close packing).  The mesh is written to a binary
    STL file and loaded from it (sd_engine_add_mesh_stl: the smooth-face rule
    recovers the wall and the two caps).  Unless `tune` is off, the
    autotuner picks the contact-list skin on the warmed-up drum, timing each
    by the mean over 24 steps (the turning wall moves spheres out of their
    skins, so list builds recur and must count).  Device time per step, CUDA
    events, a 256 MB write before every timed step."""
    import torch
    import stardust_gb300 as sd
    from stardust_gb300 import scenes
    t0 = time.perf_counter()
    d = scenes.drum_scene()
    gen_s = time.perf_counter() - t0
    d["cfg"].cuda_device = local
    eng = sd.DEMEngine(d["cfg"])
    with tempfile.TemporaryDirectory() as td:  # the mesh goes through a binary STL file (DEMMesh's route)
        scenes.add_drum_scene(eng, d, stl_path=Path(td) / "drum.stl")
    eng.prepare()
    dt = d["dt"]
    eng.step(dt, warmup)
    eng.sync()
    tuned = None
    from stardust_gb300 import _abi
    skin_before = _abi.tune_get("skin_um")
    if tune:  # the contact-list skin, timed by the mean over 24 steps (the turning wall makes builds recur)
        from stardust_gb300 import autotune
        tuned = autotune.tune_engine(eng, dt, reps=24, knobs={"skin_um": (50, 100, 200, 400, 800, 1600)},
                                     rounds=1, label="drum", stat="mean")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    st = torch.cuda.ExternalStream(eng.stream(), device=torch.device("cuda", local))
    a = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    b = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for i in range(steps):
        with torch.cuda.stream(st):
            flush.fill_(i & 0xFF)
        a[i].record(st)
        eng.step(dt, 1)
        b[i].record(st)
    torch.cuda.synchronize()
    ms = sum(x.elapsed_time(y) for x, y in zip(a, b)) / steps
    stt = eng.stats()
    n = eng.n
    eng.close()
    # the same drum with the triangles' sweep and prune along the drum axis
    # (collision engine SAP) in place of the mesh grid
    d["cfg"].collision_engine = _abi.SD_ENGINE_SAP
    eng = sd.DEMEngine(d["cfg"])
    scenes.add_drum_scene(eng, d)
    eng.prepare()
    eng.step(dt, 3)
    eng.sync()
    st2 = torch.cuda.ExternalStream(eng.stream(), device=torch.device("cuda", local))
    k = 5
    a2, b2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a2.record(st2)
    eng.step(dt, k)
    b2.record(st2)
    torch.cuda.synchronize()
    sap_ms = a2.elapsed_time(b2) / k
    sap_err = eng.stats()["device_errors"]
    eng.close()
    _abi.tune_set("skin_um", skin_before)
    return {"ms_per_step_sap_triangles": sap_ms, "device_errors_sap": sap_err,
            "workload": f"rotating drum, {n} spheres ({len(d['clumps'])} 4-sphere clumps), "
                        f"{len(d['tris'])} triangles loaded from a binary STL, R 0.5 m, L 0.5 m, 2 rad/s, dt 2e-6 s",
            "spheres": n, "bodies": int(stt["n_bodies"]), "triangles": int(len(d["tris"])), "ms_per_step": ms,
            "particle_steps_per_s": n / (ms * 1e-3), "device_errors": stt["device_errors"],
            "moved_keys_last_step": stt["moved_keys"], "list_builds": stt["list_builds"],
            "listed_steps": stt["listed_steps"], "scene_generation_s": gen_s, "autotune": tuned}


def bench_sap(n: int, steps: int, warmup: int, local: int):
    """The sweep-and-prune operators on n boxes (centres uniform in the unit
    cube, half-width 2.5 mm, seeded) -- SAPCollision::processCollisions's
    bug-compatible rows (sd_sap_process_collisions: boxes, stable sort of the
    lower x, windowed sweep) and the exact pair set (sd_sap_pairs).  The
    reference records 6.8-8.6 ms per "blocksweep"/"serialweep" run
    (profiling/*.txt) for testSAP.cu, whose setup is 2,000,000 objects but
    whose hardware and initialisation are not recorded.  The exact sweep is
    binned into y-z columns (each box sweeps only the boxes of its own
    columns); the LBVH operator (sd_lbvh_pairs) gives the same pair set.
    CUDA events on the current stream, mean over `steps` calls after
    `warmup` (each call includes its scratch allocation from torch's cache
    and the read of the pair count)."""
    import torch
    import stardust_gb300 as sd
    g = torch.Generator(device="cpu").manual_seed(7)
    pos = torch.empty((n, 4), dtype=torch.float32)
    pos[:, :3] = torch.rand((n, 3), generator=g)
    pos[:, 3] = 0.0025
    pos = pos.to(f"cuda:{local}")
    lo = (pos[:, :3] - pos[:, 3:]).contiguous()
    hi = (pos[:, :3] + pos[:, 3:]).contiguous()
    lo4 = torch.cat([lo, torch.zeros((n, 1), device=lo.device)], 1).contiguous()
    hi4 = torch.cat([hi, torch.zeros((n, 1), device=hi.device)], 1).contiguous()
    cap = 1 << 24
    out = {"workload": f"{n} boxes, centres uniform in the unit cube, half-width 2.5 mm"}
    for name, fn in (("process_collisions_ms", lambda: sd.SweepAndPrune.process_collisions(pos)),
                     ("exact_pairs_ms", lambda: sd.SweepAndPrune.pairs(lo4, hi4, cap)),
                     ("lbvh_pairs_ms", lambda: sd.BoundingVolumes.pairs(lo4, hi4, cap))):
        for _ in range(warmup):
            r = fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            r = fn()
        b.record()
        torch.cuda.synchronize()
        out[name] = a.elapsed_time(b) / steps
        if name != "process_collisions_ms":
            out[name.replace("_ms", "_count")] = int(r[1])
    out["reference_recorded_ms"] = {"blocksweep_median": 7.048, "serialweep_median": 7.054}
    return out


def timed_steps(eng, dt: float, k: int, stream, flush) -> list:
    """k steps, each after a 256 MB write that flushes the L2, one CUDA event
    pair per step on the engine's stream: the per-step device times (ms)."""
    import torch
    a = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
    b = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
    for i in range(k):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xFF)
        a[i].record(stream)
        eng.step(dt, 1)
        b[i].record(stream)
    torch.cuda.synchronize()
    return [x.elapsed_time(y) for x, y in zip(a, b)]


def autotune_table() -> dict:
    """The launch knobs chosen per size bucket in this run."""
    from stardust_gb300 import autotune
    return autotune.table()


def with_knobs(knobs: dict, fn):
    """Runs fn() with launch knobs set, then restores them."""
    from stardust_gb300 import _abi
    old = {k: _abi.tune_get(k) for k in knobs}
    try:
        for k, v in knobs.items():
            _abi.tune_set(k, v)
        return fn()
    finally:
        for k, v in old.items():
            _abi.tune_set(k, v)


def bench_dense_bed(pos, vel, cfg, dt, steps: int, advance: int, local: int, tune: bool):
    """The same 1,048,576 spheres with radii inflated by 1.2: an overlapping
    contact network of ~2.5M pairs, advanced `advance` steps (the explosive
    start relaxes), the contact-list skin chosen by the autotuner on that
    state, then `steps` device-timed steps (L2 flushed before each), with
    and without contact lists."""
    import torch
    import stardust_gb300 as sd
    p = pos.copy()
    p[:, 3] *= np.float32(1.2)
    c = sd.EngineConfig(**{**cfg.__dict__})
    c.cell = float(2 * p[:, 3].max())
    c.cuda_device = local
    eng = sd.DEMEngine(c)
    eng.add_spheres(p, vel)
    eng.prepare()
    stream = torch.cuda.ExternalStream(eng.stream(), device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    from stardust_gb300 import _abi, autotune
    eng.step(dt, advance)
    old = {k: _abi.tune_get(k) for k in ("skin_um", "listed_blocks")}
    tuned = None
    if tune:  # the skin and the list kernel's register budget, for this contact network
        tuned = autotune.tune_engine(eng, dt, reps=3, knobs={"skin_um": (0, 50, 200, 500), "listed_blocks": (4, 5, 6)},
                                     label=autotune.bucket_of(eng) + ":dense")
    skin = _abi.tune_get("skin_um")
    eng.step(dt, 3)
    ms = statistics.mean(timed_steps(eng, dt, steps, stream, flush))
    no_lists = statistics.mean(with_knobs({"skin_um": 0}, lambda: timed_steps(eng, dt, steps, stream, flush)))
    for k, v in old.items():
        _abi.tune_set(k, v)
    st = eng.stats()
    eng.close()
    n = len(p)
    return {"workload": f"{n} spheres of the settling box with radii x1.2, after {advance} steps",
            "contacts": st["contacts"], "ms_per_step": ms, "particle_steps_per_s": n / (ms * 1e-3),
            "skin_um": skin, "ms_per_step_without_contact_lists": no_lists,
            "moved_keys_last_step": st["moved_keys"], "device_errors": st["device_errors"],
            "autotune": None if tuned is None else tuned["choice"]}


def run_ours(args, rank, world, local):
    import torch
    import torch.distributed as dist
    import stardust_gb300 as sd
    from stardust_gb300 import _abi

    torch.cuda.set_device(local)
    if world > 1 and not dist.is_initialized():
        dist.init_process_group("nccl")
    n = args.n
    pos, vel, cfg, dt, phi = build_scene(n, args.seed + rank)
    cfg.cuda_device = local
    cfg.flags = 0
    eng = sd.DEMEngine(cfg)
    eng.add_spheres(pos, vel)
    eng.prepare()
    stream = torch.cuda.ExternalStream(eng.stream(), device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    # the first steps after the packing (graph capture happens on the first
    # step): a short window kept as an extra key
    eng.step(dt, args.warmup)
    eng.sync()
    early_ms = statistics.mean(timed_steps(eng, dt, 10, stream, flush))
    early = eng.stats()
    # the timed window lies inside the config's 2,000-step settling run: the
    # scene is advanced (untimed) to step `advance` first, then the
    # autotuner picks the launch knobs on that state (its steps advance the
    # run too), then warm-up
    eng.step(dt, max(0, args.advance - int(early["steps"])))
    eng.sync()
    tuned = None
    if not args.no_tune:
        from stardust_gb300 import autotune
        tuned = autotune.tune_engine(eng, dt, reps=5)
        log(f"autotune: {tuned}")
    # the knobs this workload is timed with (later sections tune their own)
    knobs = {k: _abi.tune_get(k) for k in ("contact_mode", "sort_items", "z_div", "resort_max", "pair_lists",
                                           "skin_um")}
    eng.step(dt, args.warmup)
    eng.sync()
    first_step = int(eng.stats()["steps"]) + 1

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-timed steps (value)
    barrier()
    with Clocks(local) as clk:
        step_ms = timed_steps(eng, dt, args.steps, stream, flush)
        barrier()
    clocks = clk.summary()
    eng.sync()
    st = eng.stats()
    from stardust_gb300 import replicas
    total_ms = replicas.max_over_ranks(sum(step_ms), device=f"cuda:{local}")
    value = replicas.job_rate(n * args.steps, total_ms * 1e-3, device=f"cuda:{local}")
    window = {"first_step": first_step, "last_step": int(st["steps"]), "contacts": st["contacts"],
              "moved_keys_last_step": st["moved_keys"], "list_builds": st["list_builds"],
              "listed_steps": st["listed_steps"]}

    # ---- the same state without the contact lists, and with the full radix
    # sort every step (no incremental re-sort, hence no lists either)
    k_cmp = max(10, args.steps // 2)
    no_lists_ms = statistics.mean(with_knobs({"skin_um": 0}, lambda: timed_steps(eng, dt, k_cmp, stream, flush)))
    full_sort_ms = statistics.mean(with_knobs({"resort_max": 0},
                                              lambda: timed_steps(eng, dt, k_cmp, stream, flush)))
    eng.step(dt, 2)  # the step graph of the timed knobs again (the stages below run its variant)
    eng.sync()

    # ---- dominant kernel alone: contact + integrate (idempotent stage: the
    # step's own variant, i.e. the listed contacts between list builds)
    kstarts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stage_ms = {}
    # the stage API's stages, each timed alone: the step graph runs the
    # contact stage as is, but replaces the full radix sort and the gather
    # reorder with the incremental re-sort and the in-place reorder when few
    # cell keys changed (stages_note in the JSON line)
    for name, stage in (("contact_integrate", _abi.SD_STAGE_CONTACT), ("radix_sort", _abi.SD_STAGE_SORT),
                        ("gather_reorder", _abi.SD_STAGE_REORDER)):
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
            kstarts[k].record(stream)
            _abi.call("sd_engine_launch_stage", eng._h, stage, dt, h=eng._h)
            kends[k].record(stream)
        torch.cuda.synchronize()
        ms = [s.elapsed_time(e) for s, e in zip(kstarts, kends)]
        stage_ms[name] = sum(ms) / len(ms)
    eng.sync()
    contact_ms = stage_ms["contact_integrate"]
    lists_on = knobs["skin_um"] > 0 and knobs["resort_max"] > 0 and knobs["contact_mode"] == 0
    contact_bytes = CONTACT_BYTES_PER_SPHERE + (LIST_BYTES_PER_SPHERE if lists_on else 0)
    peak, peak_kind = measured_peak()
    achieved = n * contact_bytes / (contact_ms * 1e-3) / 1e9
    traffic_ps, winst_ps = recorded_profile("listed" if lists_on else "scan")

    # ---- end to end through the C ABI with host buffers: the host owns the
    # state; every step uploads positions and velocities from pinned memory,
    # steps, and reads the new positions and velocities back into the same
    # buffers (the next step's inputs)
    hpos = torch.from_numpy(eng.positions()).pin_memory()
    hvel = torch.from_numpy(eng.velocities()).pin_memory()
    import ctypes as C
    lib = _abi.lib()
    nbytes = hpos.numel() * 4

    def host_step():
        _abi.check(lib.sd_engine_set_state(eng._h, _abi.SD_FIELD_POSITION, C.c_void_p(hpos.data_ptr()), nbytes),
                   "set_state", eng._h)
        _abi.check(lib.sd_engine_set_state(eng._h, _abi.SD_FIELD_VELOCITY, C.c_void_p(hvel.data_ptr()), nbytes),
                   "set_state", eng._h)
        _abi.check(lib.sd_engine_step(eng._h, dt, 1), "step", eng._h)
        _abi.check(lib.sd_engine_get_state(eng._h, _abi.SD_FIELD_POSITION, C.c_void_p(hpos.data_ptr()), nbytes),
                   "get_state", eng._h)
        _abi.check(lib.sd_engine_get_state(eng._h, _abi.SD_FIELD_VELOCITY, C.c_void_p(hvel.data_ptr()), nbytes),
                   "get_state", eng._h)

    host_step()  # untimed: the stage timing above left the engine to re-sort once
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        host_step()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e = replicas.job_rate(n * args.steps, e2e_s, device=f"cuda:{local}")
    eng.close()

    # ---- a dense contact network of the same spheres (rank 0, N = 1)
    dense = None
    if rank == 0 and world == 1 and not args.no_dense:
        dense = bench_dense_bed(pos, vel, cfg, dt, 20, 1000, local, not args.no_tune)
        log(f"dense bed: {dense}")

    # ---- learned GJK warm start on the convex-hull step (rank 0, N = 1)
    gjk = None
    if rank == 0 and world == 1 and not args.no_hulls:
        gjk = bench_hulls(args.hulls, 20, 100, local)
        log(f"gjk: {gjk}")

    # ---- batched scenes (rank 0, N = 1)
    batch = None
    if rank == 0 and world == 1 and not args.no_batch:
        batch = bench_batch(args.scenes, args.steps, args.warmup, local, not args.no_tune)
        log(f"batch: {batch}")

    # ---- rotating drum (rank 0, N = 1)
    drum = None
    if rank == 0 and world == 1 and not args.no_drum:
        drum = bench_drum(args.steps, args.warmup, local, not args.no_tune)
        log(f"drum: {drum}")

    # ---- sweep and prune on 2,000,000 boxes (rank 0, N = 1)
    sap = None
    if rank == 0 and world == 1 and not args.no_sap:
        sap = bench_sap(2_000_000, 20, 3, local)
        log(f"sap: {sap}")

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        n_cpu = min(n, args.cpu_n)
        if n_cpu == n:
            cp, cv, ccfg, cdt = pos, vel, cfg, dt
        else:
            cp, cv, ccfg, cdt, _ = build_scene(n_cpu, args.seed)
        rate, used, csteps, cel = cpu_oracle_rate(cp, cv, ccfg, cdt, args.cpu_seconds, None, args.z_div)
        cpu = {"value": rate, "unit": UNIT, "cores": used, "kind": "port",
               "sample": f"{csteps} steps of the {n_cpu}-sphere scene in {cel:.1f}s, CPU restatement of the step "
                         f"(oracle/, OpenMP, {used} threads)"}

    # ---- the reference's own GPU step (its kernels, compiled unchanged from
    # its sources) on the same scene and GPU (rank 0, N = 1): a baseline leg
    ref_gpu = None
    if rank == 0 and world == 1 and args.ref_gpu:
        try:
            from oracle import time_ref_step
            ref_gpu = time_ref_step.measure(5, 2, n, scene=(pos, vel, dt))
        except BaseException as e:  # noqa: BLE001 -- a baseline leg never fails the bench
            ref_gpu = {"impl": "reference-gpu", "unavailable": f"{type(e).__name__}: {e}"}
        if ref_gpu.get("ms_per_step"):
            ref_gpu["ours_speedup"] = ref_gpu["ms_per_step"] / (total_ms / args.steps)
        log(f"reference GPU step: {ref_gpu}")

    if rank == 0:
        sm_mhz = clocks_mhz(clocks)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"settling box, {n} polydisperse spheres, 1x1x2 m, dt 5e-6 s, 2000-step run",
                       "n_spheres": n, "volume_fraction": round(phi, 4), "cells": st["n_cells"],
                       "timed_window": f"steps {window['first_step']}-{window['last_step']} of the run",
                       "l2": "flushed (256 MB write) before every timed step", "parallelism": f"replicas{world}",
                       "knobs": knobs},
            "timed_window": window,
            "early_window": {"steps": f"{args.warmup + 1}-{args.warmup + 10}", "ms_per_step": early_ms,
                             "contacts": early["contacts"], "moved_keys_last_step": early["moved_keys"]},
            "ms_per_step_without_contact_lists": no_lists_ms,
            "ms_per_step_full_radix_sort": full_sort_ms,
            "autotune": tuned,
            "autotune_table": None if args.no_tune else autotune_table(),
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 2 * nbytes, "d2h_bytes_per_step": 2 * nbytes},
            "roofline": {"bound": "hbm", "kernel": "dem_contact_integrate_kernel" + (" (listed)" if lists_on else ""),
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind,
                         "traffic": None if traffic_ps is None else traffic_ps * n,
                         "algorithmic_bytes": contact_bytes * n, "launch_ms": contact_ms},
            # a scan-bound contact kernel is bound by instruction issue, not
            # bytes: its warp instructions per launch (ncu) over the live
            # launch time, against one warp instruction per scheduler per clock
            "issue_roofline": None if winst_ps is None else {
                "kernel": "dem_contact_integrate_kernel", "unit": "warp instructions/s",
                "achieved": winst_ps * n / (contact_ms * 1e-3),
                "peak": SMS * SCHEDULERS_PER_SM * sm_mhz * 1e6,
                "frac": winst_ps * n / (contact_ms * 1e-3) / (SMS * SCHEDULERS_PER_SM * sm_mhz * 1e6),
                "warp_instructions": winst_ps * n, "sm_mhz": sm_mhz},
            "stages_ms": stage_ms,
            "stages_note": "sd_engine_launch_stage stages timed alone; in the step graph the radix sort and gather "
                           "reorder give way to the incremental re-sort (scan) and in-place reorder while at most "
                           "resort_max keys change",
            "step_bytes_per_sphere": STEP_BYTES_PER_SPHERE,
            "step_hbm_frac": (n * STEP_BYTES_PER_SPHERE / (total_ms / args.steps * 1e-3) / 1e9) / peak,
            "cpu_baseline": cpu,
            "reference_gpu": ref_gpu,
            "clocks": clocks,
            "gpu_launches": st["step_kernels"] * args.steps,
            "contacts": st["contacts"],
            "moved_keys_last_step": st["moved_keys"],
            "dense_bed": dense,
            "gjk": gjk,
            "batch": batch,
            "drum": drum,
            "sap": sap,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_FULL)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--cpu-n", type=int, default=N_FULL)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--advance", type=int, default=1000,
                    help="untimed steps of the settling run before tuning and timing (the timed window's start)")
    ap.add_argument("--no-dense", action="store_true", help="skip the dense contact network (radii x1.2)")
    ap.add_argument("--ref-gpu", action="store_true",
                    help="also time the reference's own GPU kernels stage by stage (oracle/time_ref_step.py)")
    # the default now; accepted so that older command lines still parse
    ap.add_argument("--no-ref-gpu", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--no-hulls", action="store_true")
    ap.add_argument("--only-hulls", action="store_true", help="run only the convex-hull GJK section")
    ap.add_argument("--hulls", type=int, default=65_536)
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--only-batch", action="store_true", help="run only the batched-scenes section")
    ap.add_argument("--scenes", type=int, default=512)
    ap.add_argument("--no-drum", action="store_true")
    ap.add_argument("--only-drum", action="store_true", help="run only the rotating-drum section")
    ap.add_argument("--no-sap", action="store_true")
    ap.add_argument("--only-sap", action="store_true", help="run only the sweep-and-prune section")
    ap.add_argument("--z-div", type=int, default=None,
                    help="z cells per cell edge for every engine (default: the library's automatic choice)")
    ap.add_argument("--knob", action="append", default=[], metavar="NAME=VALUE",
                    help="set a launch knob (sd_tune_set) before anything runs; repeatable")
    args = ap.parse_args()
    if args.z_div is not None or args.knob:
        from stardust_gb300 import _abi
        if args.z_div is not None:
            _abi.tune_set("z_div", args.z_div)
        for kv in args.knob:
            name, value = kv.split("=", 1)
            _abi.tune_set(name, int(value))
    if args.warmup < 3:
        log("warm-up raised to 3 steps (timing rule)")
        args.warmup = 3
    rank, world, local = dist_env()
    if args.only_sap:
        import torch
        torch.cuda.set_device(local)
        print(json.dumps({"sap": bench_sap(2_000_000, args.steps, args.warmup, local)}), flush=True)
        return 0
    if args.only_drum:
        import torch
        torch.cuda.set_device(local)
        print(json.dumps({"drum": bench_drum(args.steps, args.warmup, local, not args.no_tune)}), flush=True)
        return 0
    if args.only_batch:
        import torch
        torch.cuda.set_device(local)
        print(json.dumps({"batch": bench_batch(args.scenes, args.steps, args.warmup, local, not args.no_tune)}),
              flush=True)
        return 0
    if args.only_hulls:
        import torch
        torch.cuda.set_device(local)
        print(json.dumps({"gjk": bench_hulls(args.hulls, args.steps, args.warmup, local)}), flush=True)
        return 0
    if args.impl == "reference":
        return run_reference_arm(args, rank, world)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
