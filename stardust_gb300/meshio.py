"""STL meshes: read (through the library's reader), smooth-face patches, and
write (binary or ASCII) -- the mesh side of a scene, for sd_engine_add_mesh /
sd_engine_add_mesh_stl and for the JSON scene's "mesh" entities."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _abi


def read_stl(path) -> np.ndarray:
    """Triangles of an ASCII or binary STL file as an (n, 3, 3) float32 array
    (sd_stl_read)."""
    n = C.c_uint64()
    _abi.check(_abi.lib().sd_stl_read(str(path).encode(), 0, None, C.byref(n)), "sd_stl_read")
    out = np.empty((n.value, 3, 3), np.float32)
    _abi.check(_abi.lib().sd_stl_read(str(path).encode(), n.value, out.ctypes.data, C.byref(n)), "sd_stl_read")
    return out


def mesh_patches(tris, angle_deg: float = 30.0) -> np.ndarray:
    """Smooth-face ids (sd_mesh_patches): triangles sharing an edge whose
    normals (as unoriented lines) differ by less than angle_deg share an id."""
    t = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    out = np.empty(len(t), np.int32)
    _abi.check(_abi.lib().sd_mesh_patches(len(t), t.ctypes.data, angle_deg, out.ctypes.data), "sd_mesh_patches")
    return out


def _normals(t: np.ndarray) -> np.ndarray:
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]).astype(np.float64)
    l = np.linalg.norm(n, axis=1, keepdims=True)
    return np.where(l > 0, n / np.where(l > 0, l, 1), 0).astype(np.float32)


def write_stl(path, tris, binary: bool = True, name: str = "stardust") -> None:
    """Writes (n, 3, 3) triangles as an STL file.  ASCII coordinates use 9
    significant digits, so float32 values read back exactly."""
    t = np.ascontiguousarray(tris, np.float32).reshape(-1, 3, 3)
    nrm = _normals(t)
    path = Path(path)
    if binary:
        rec = np.zeros(len(t), dtype=[("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")])
        rec["n"] = nrm
        rec["v"] = t
        with open(path, "wb") as f:
            f.write(name.encode()[:80].ljust(80, b" "))
            f.write(np.uint32(len(t)).tobytes())
            f.write(rec.tobytes())
        return
    lines = [f"solid {name}"]
    for tri, n in zip(t, nrm):
        lines.append("  facet normal {:.9g} {:.9g} {:.9g}".format(*n))
        lines.append("    outer loop")
        for v in tri:
            lines.append("      vertex {:.9g} {:.9g} {:.9g}".format(*v))
        lines.append("    endloop")
        lines.append("  endfacet")
    lines.append(f"endsolid {name}")
    path.write_text("\n".join(lines) + "\n")
