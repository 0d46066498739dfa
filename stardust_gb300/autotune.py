"""Launch-knob autotuner.

The reference picks block sizes by hand-run sweeps whose wall times it keeps
in profiling/blocksweep*.txt (averaged by profiling/profile_1.py).  Here the
engine's own step is timed on the device for every combination of the
process-wide knobs (``sd_tune_set``: contact-scan variant, sort tile size),
with the L2 flushed before each timed step, and the fastest combination is
kept.  Tuning steps advance the simulation like any other step.
"""
from __future__ import annotations

import itertools

from . import _abi

KNOBS = {"contact_mode": (0, 1), "sort_items": (8, 16), "skin_um": (0, 20, 50, 100, 200), "listed_blocks": (4, 5)}
# a batch of scenes takes no contact lists; its pair lists are a choice
BATCH_KNOBS = {"sort_items": (8, 16), "pair_lists": (0, 2)}


def tune_engine(eng, dt: float, reps: int = 5, knobs: dict | None = None, flush_bytes: int = 256 << 20) -> dict:
    """Time `reps` steps per knob combination; set and return the best."""
    import torch

    knobs = knobs or KNOBS
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.ExternalStream(eng.stream(), device=dev)
    flush = torch.empty(flush_bytes, dtype=torch.uint8, device=dev)
    names = list(knobs)
    table = []
    for combo in itertools.product(*(knobs[k] for k in names)):
        c = dict(zip(names, combo))
        # combinations that run the same kernels as one already timed: the
        # column kernel takes no contact lists, and the list kernel's
        # register cap matters only with lists
        if c.get("contact_mode", 0) == 1 and (c.get("skin_um", 0) != 0 or c.get("listed_blocks", 4) != 4):
            continue
        if c.get("skin_um", 1) == 0 and c.get("listed_blocks", 4) != 4:
            continue
        for k, v in zip(names, combo):
            _abi.tune_set(k, v)
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
        table.append({"knobs": dict(zip(names, combo)), "ms_median": ms[len(ms) // 2]})
    best = min(table, key=lambda r: r["ms_median"])
    for k, v in best["knobs"].items():
        _abi.tune_set(k, v)
    eng.step(dt, 1)
    eng.sync()
    return {"choice": best["knobs"], "table": table}
