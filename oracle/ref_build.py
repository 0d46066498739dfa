"""Builds the reference's own kernels for pinning the oracle (test infrastructure).

* ``build_cubins()`` compiles the reference kernel sources, unchanged and
  where they lie under the reference checkout (``STARDUST_REF`` or
  /root/reference), into sm_103a cubins in ``oracle/_ref/``.  The only
  addition is ``oracle/ref_shim/ref_types_shim.h``: the include guards of the
  reference's engine.hpp and types.hpp are pre-defined (those headers pull
  Eigen and OpenGL) and the two names the kernels use from them, ``Scalar``
  and ``float9``, are declared.  Needs the reference checkout, so it runs in
  the build container; the cubins travel with the repository copy.
* ``build_sandbox_cubins()`` does the same for the LBVH and GJK prototypes
  (``sandbox/testLBVH.cu``, ``sandbox/testGJK.cu``), which do not compile as
  written: it copies the sandbox sources into ``oracle/_ref/sandbox/``
  (git-ignored, never committed, removed after the compile) and applies the
  edits listed in
  ``SANDBOX_EDITS`` -- an include guard for ``util.hpp``, ``const`` on the
  support functions' direction parameter (the calls at testGJK.cu:106,110,114
  pass ``-direction``, a temporary), ``void main`` renamed (it is not a
  kernel), and testLBVH.cu's ``#include "testGJK.cu"`` dropped (the Morton
  kernel does not use it) -- plus ``oracle/ref_shim/sandbox_shim.h``, the
  unary minus on ``float3`` that testGJK.cu:279 uses and helper_math.hpp
  lacks.  The kernels themselves are unchanged.
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


SANDBOX_FILES = ("testLBVH.cu", "testGJK.cu", "cuda_utils.hpp", "helper_math.hpp", "util.hpp", "primitives.hpp",
                 "types.hpp")
# (file, regular expression, replacement, expected number of matches)
SANDBOX_EDITS = (
    ("util.hpp", r"\A", "#pragma once\n", 1),
    ("testGJK.cu", r"(supportSphere\(\s*)float4& direction", r"\1const float4& direction", 1),
    ("testGJK.cu", r"(supportPointSoupNaive\(\s*)float4& direction", r"\1const float4& direction", 1),
    ("testGJK.cu", r"\bvoid main\(\)", "int sandbox_gjk_main()", 1),
    ("testLBVH.cu", r'#include "testGJK\.cu"\n', "", 1),
)
SANDBOX_CUBINS = ("testLBVH", "testGJK")


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


def build_sandbox_cubins(verbose: bool = False) -> bool:
    """The LBVH/GJK prototypes' cubins, from edited copies (see the module
    docstring); True when they exist afterwards."""
    import re
    ref = reference_root()
    have = all((OUT / f"{s}.cubin").exists() for s in SANDBOX_CUBINS)
    if ref is None or not (ref / "sandbox").is_dir():
        return have
    work = OUT / "sandbox"
    work.mkdir(parents=True, exist_ok=True)
    newest = max((ref / "sandbox" / f).stat().st_mtime for f in SANDBOX_FILES)
    newest = max(newest, Path(__file__).stat().st_mtime, (HERE / "ref_shim" / "sandbox_shim.h").stat().st_mtime)
    if have and all((OUT / f"{s}.cubin").stat().st_mtime >= newest for s in SANDBOX_CUBINS):
        return True
    for f in SANDBOX_FILES:
        text = (ref / "sandbox" / f).read_text()
        for name, pat, rep, count in SANDBOX_EDITS:
            if name == f:
                text, k = re.subn(pat, rep, text)
                if k != count:
                    sys.stderr.write(f"sandbox edit {pat!r} matched {k} times in {f}\n")
                    return False
        (work / f).write_text(text)
    for s in SANDBOX_CUBINS:
        cmd = [_nvcc(), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-w",
               "-include", str(HERE / "ref_shim" / "sandbox_shim.h"), "-o", str(OUT / f"{s}.cubin"),
               str(work / f"{s}.cu")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            return False
    shutil.rmtree(work, ignore_errors=True)  # the edited copies are only an input of the cubins
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
    print("sandbox cubins:", build_sandbox_cubins(verbose=True))
    print("harness:", build_harness(verbose=True))
