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
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRCS = [HERE / "sd_oracle.c", HERE / "sd_oracle_hull.c"]


def build(verbose: bool = False) -> Path:
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle")
    deps = SRCS + [HERE / "sd_oracle.h", Path(__file__)]
    if LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    cmd = [cc, "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", "-o", str(LIB)] + [str(s) for s in SRCS] + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
