"""Launch-knob autotuner, per size bucket.

The reference picks block sizes by hand-run sweeps whose wall times it keeps
in profiling/blocksweep*.txt (averaged by profiling/profile_1.py).  Here the
engine's own step is timed on the device, the L2 flushed before every timed
step, over the process-wide launch knobs (``sd_tune_set``): the contact
stage's variant and launch shape (per-sphere kernel or column tiles, threads
per block, the contact-list skin and the list kernel's register cap), the
sort's tile size, the re-sort's limit, the pair lists of a batch and the
reorder's grid.  The search is coordinate descent -- every value of one knob
with the others held, knob after knob, two rounds -- from the current
settings, so a knob that interacts with another is revisited once the other
has moved.  Combinations that run the same kernels as one already timed are
skipped.

Choices are kept per size bucket: the engine's kind (one scene, or a batch
of scenes) and its sphere count in powers of eight from 4,096.  ``apply``
sets the knobs of an engine's bucket when one was tuned; ``save``/``load``
keep the table in a JSON file.  Tuning steps advance the simulation like any
other step.
"""
from __future__ import annotations

import json
import math

from . import _abi

SCENE_KNOBS = {"skin_um": (0, 20, 50, 100, 200), "listed_blocks": (4, 5, 6), "contact_block": (128, 256),
               "contact_mode": (0, 1), "sort_items": (8, 16), "resort_max": (256, 1024), "fix_blocks": (4, 8)}
BATCH_KNOBS = {"skin_um": (0, 20, 50, 100), "listed_blocks": (4, 5), "contact_block": (128, 256),
               "pair_lists": (0, 2), "sort_items": (8, 16), "resort_max": (256, 1024), "fix_blocks": (4, 8)}

_TABLE: dict[str, dict] = {}


def bucket_of(eng) -> str:
    """'scene' or 'batch', and the sphere count rounded down to a power of
    eight (at least 4,096): e.g. 'scene:2^18' holds 262,144-2,097,151."""
    n = max(int(eng.n), 1)
    kind = "batch" if getattr(eng, "n_scenes", 0) > 1 else "scene"
    e = max(12, 3 * int(math.log(n, 8)))
    return f"{kind}:2^{e}"


def _redundant(c: dict) -> bool:
    """Knob settings that run the same kernels as a setting already timed."""
    if c.get("contact_mode", 0) == 1 and (c.get("skin_um", 0) != 0 or c.get("listed_blocks", 5) != 5
                                         or c.get("contact_block", 256) != 256):
        return True  # the column kernel takes no lists and has its own shape
    if c.get("skin_um", 1) == 0 and c.get("listed_blocks", 5) != 5:
        return True  # the register cap belongs to the list kernel
    if c.get("resort_max", 1) == 0 and c.get("skin_um", 0) != 0:
        return True  # no lists without the re-sort
    return False


def _time(eng, dt: float, reps: int, stream, flush, stat: str = "median") -> float:
    import torch
    eng.step(dt, 2)  # re-capture + warm
    eng.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for a, b in ev:
        with torch.cuda.stream(stream):
            flush.fill_(1)
        a.record(stream)
        eng.step(dt, 1)
        b.record(stream)
    torch.cuda.synchronize()
    ms = sorted(a.elapsed_time(b) for a, b in ev)
    return sum(ms) / len(ms) if stat == "mean" else ms[len(ms) // 2]


def tune_engine(eng, dt: float, reps: int = 5, knobs: dict | None = None, rounds: int = 2,
                flush_bytes: int = 256 << 20, label: str | None = None, stat: str = "median",
                timer=None) -> dict:
    """Coordinate descent over `knobs` (default: the bucket kind's set) on
    the live engine; sets the best and records it for the engine's bucket
    (or under `label`, for a regime of one bucket tuned apart, e.g. a dense
    bed).  Each setting is timed over `reps` steps by their median, or by
    their mean (stat "mean": for scenes whose contact-list builds recur
    within a few steps, e.g. a turning drum, so that the builds count).
    `timer` (tests): a function of no arguments that times the current
    settings in its place.  Returns {"bucket", "choice", "ms", "table"}:
    every timed setting."""
    bucket = label or bucket_of(eng)
    if knobs is None:
        knobs = BATCH_KNOBS if bucket.startswith("batch") else SCENE_KNOBS
    if timer is None:
        import torch

        dev = torch.device("cuda", torch.cuda.current_device())
        stream = torch.cuda.ExternalStream(eng.stream(), device=dev)
        flush = torch.empty(flush_bytes, dtype=torch.uint8, device=dev)

        def timer():
            return _time(eng, dt, reps, stream, flush, stat)
    cur = {k: _abi.tune_get(k) for k in knobs}
    seen: dict[tuple, float] = {}
    table = []

    def run(c: dict) -> float:
        key = tuple(sorted(c.items()))
        if key not in seen:
            for k, v in c.items():
                _abi.tune_set(k, v)
            seen[key] = timer()
            table.append({"knobs": dict(c), f"ms_{stat}": seen[key]})
        return seen[key]

    best_ms = run(cur)
    for _ in range(rounds):
        moved = False
        for k, values in knobs.items():
            for v in values:
                c = dict(cur, **{k: v})
                if c == cur or _redundant(c):
                    continue
                ms = run(c)
                if ms < best_ms:
                    best_ms, cur, moved = ms, c, True
        if not moved:
            break
    for k, v in cur.items():
        _abi.tune_set(k, v)
    eng.step(dt, 1)
    eng.sync()
    _TABLE[bucket] = dict(cur)
    return {"bucket": bucket, "choice": dict(cur), "ms": best_ms, "table": table}


def apply(eng) -> dict | None:
    """Sets the knobs tuned for the engine's bucket (None when none was)."""
    c = _TABLE.get(bucket_of(eng))
    if c:
        for k, v in c.items():
            _abi.tune_set(k, v)
    return c


def table() -> dict:
    """The per-bucket choices tuned so far in this process."""
    return {k: dict(v) for k, v in _TABLE.items()}


def save(path) -> None:
    with open(path, "w") as f:
        json.dump(_TABLE, f, indent=1, sort_keys=True)


def load(path) -> dict:
    with open(path) as f:
        _TABLE.update(json.load(f))
    return table()
