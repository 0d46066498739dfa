"""Builds the CPU oracle (test infrastructure only).

``oracle/liboracle.so`` is the plain-C restatement in sd_oracle.c and
sd_oracle_hull.c, compiled
with -ffp-contract=off so each float operation rounds once (matching the
-fmad=false CUDA kernels).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU legs load it.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRCS = [HERE / "sd_oracle.c", HERE / "sd_oracle_hull.c"]
# the seeded scene builders, shared with the library so that both sides of a
# comparison draw the same inputs; compiled here as plain C++ under sdo_ names
SCENES = HERE.parent / "stardust_gb300" / "csrc" / "sd_scenes.cu"


def build(verbose: bool = False) -> Path:
    cc = shutil.which("gcc") or shutil.which("cc")
    cxx = shutil.which("g++") or shutil.which("c++")
    if cc is None or cxx is None:
        raise RuntimeError("no C/C++ compiler for the oracle")
    deps = SRCS + [SCENES, HERE / "sd_oracle.h", HERE.parent / "include" / "stardust.h", Path(__file__)]
    if LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    with tempfile.TemporaryDirectory() as td:
        obj = Path(td) / "sd_scenes.o"
        steps = [
            [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-DSD_SCENES_STANDALONE",
             "-x", "c++", "-c", str(SCENES), "-o", str(obj)],
            [cc, "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
             "-o", str(LIB)] + [str(s) for s in SRCS] + [str(obj), "-lstdc++", "-lm"],
        ]
        for cmd in steps:
            r = subprocess.run(cmd, capture_output=True, text=True)
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("oracle build failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
