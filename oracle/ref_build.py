"""Builds the reference's own kernels for pinning the oracle (test infrastructure).

* ``build_cubins()`` compiles the reference kernel sources, unchanged and
  where they lie under the reference checkout (``STARDUST_REF`` or
  /root/reference), into sm_103a cubins in ``oracle/_ref/``.  The only
  addition is ``oracle/ref_shim/ref_types_shim.h``: the include guards of the
  reference's engine.hpp and types.hpp are pre-defined (those headers pull
  Eigen and OpenGL) and the two names the kernels use from them, ``Scalar``
  and ``float9``, are declared.  Needs the reference checkout, so it runs in
  the build container; the cubins travel with the repository copy.
* ``build_harness()`` compiles ``oracle/ref_harness.cpp`` (driver-API
  loader/launcher) into ``oracle/_ref/libref_harness.so``; runs anywhere with
  the CUDA toolkit.

Outputs go only to ``oracle/_ref/`` (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SOURCES = {"sh_collision_detection": "src/engine/cuda/sh_collision_detection.cu",
           "collision_resolution": "src/engine/cuda/collision_resolution.cu",
           "physics_update": "src/engine/cuda/physics_update.cu",
           "sap_detection": "src/engine/cuda/collisions/SAP/sap_detection.cu"}


def reference_root() -> Path | None:
    p = Path(os.environ.get("STARDUST_REF", "/root/reference"))
    return p if (p / "src" / "engine" / "cuda").is_dir() else None


def _nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build_cubins(verbose: bool = False) -> bool:
    ref = reference_root()
    if ref is None:
        return all((OUT / f"{s}.cubin").exists() for s in SOURCES)
    OUT.mkdir(exist_ok=True)
    for s, rel in SOURCES.items():
        src = ref / rel
        dst = OUT / f"{s}.cubin"
        if dst.exists() and dst.stat().st_mtime >= src.stat().st_mtime:
            continue
        cmd = [_nvcc(), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
               "-D_STARDUST_ENGINE_HEADER_", "-D_STARDUST_SIMULATION_TYPES_HEADER_",
               "-include", str(HERE / "ref_shim" / "ref_types_shim.h"), "-w", "-o", str(dst), str(src)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            return False
    return True


def build_harness(verbose: bool = False) -> Path | None:
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libref_harness.so"
    src = HERE / "ref_harness.cpp"
    if lib.exists() and lib.stat().st_mtime >= src.stat().st_mtime:
        return lib
    cuda = Path(_nvcc()).resolve().parent.parent
    cmd = [shutil.which("g++") or "g++", "-O2", "-shared", "-fPIC", "-std=c++17", f"-I{cuda / 'include'}",
           "-o", str(lib), str(src), f"-L{cuda / 'lib64'}", f"-L{cuda / 'lib64' / 'stubs'}", "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or r.returncode:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    return lib if r.returncode == 0 else None


if __name__ == "__main__":
    print("cubins:", build_cubins(verbose=True))
    print("harness:", build_harness(verbose=True))
