"""Python mirror of the reference engine surface, over the C ABI.

``DEMEngine`` follows STARDUST::DEMEngine (src/engine/engine.hpp:37-447):
``add`` / ``prep`` / ``transfer`` / ``update(dt)`` keep their meaning;
``add_spheres`` and ``step(dt, n)`` are the bulk forms.  ``SpatialPartition``
follows the static operator class of the same name
(src/engine/cuda/collision_detection.cuh:30-66) and works on CUDA tensors.
Every call goes to libstardust_gb300.so; nothing runs on the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import call, lib


@dataclass
class EngineConfig:
    """sd_config: defaults are the 4,096-sphere box config's material."""
    collision_engine: int = _abi.SD_ENGINE_SHP
    device: int = _abi.SD_DEVICE_GPU
    cuda_device: int = 0
    domain: float = 1.0
    box_lo: tuple = (0.0, 0.0, 0.0)
    box_hi: tuple = (0.0, 0.0, 0.0)
    walls: int = 0x3F
    cell: float = 0.0
    kn: float = 1e5
    restitution: float = 0.5
    mu: float = 0.3
    gravity: tuple = (0.0, 0.0, -9.81)
    pair_capacity: int = 1 << 20
    flags: int = 0

    def to_c(self) -> _abi.SdConfig:
        c = _abi.SdConfig()
        call("sd_config_default", C.byref(c))
        c.collision_engine = self.collision_engine
        c.device = self.device
        c.cuda_device = self.cuda_device
        c.domain = self.domain
        for a in range(3):
            c.box_lo[a] = self.box_lo[a]
            c.box_hi[a] = self.box_hi[a]
            c.gravity[a] = self.gravity[a]
        c.walls = self.walls
        c.cell = self.cell
        c.kn = self.kn
        c.restitution = self.restitution
        c.mu = self.mu
        c.pair_capacity = self.pair_capacity
        c.flags = self.flags
        return c


def _f32(a, cols=4) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != cols:
        raise ValueError(f"expected an (n, {cols}) float32 array, got {a.shape}")
    return a


class DEMEngine:
    """Owning handle over one sd_engine."""

    def __init__(self, config: EngineConfig | None = None):
        self.config = config or EngineConfig()
        self._c = self.config.to_c()
        h = C.c_void_p()
        call("sd_engine_create", C.byref(self._c), C.byref(h))
        self._h = h
        self._n = 0

    # -- lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().sd_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _call(self, name, *args):
        call(name, self._h, *args, h=self._h)

    # -- scene (engine.hpp:187-190)
    def add_spheres(self, pos4, vel4, omega4=None) -> None:
        p = _f32(pos4)
        v = _f32(vel4)
        if len(p) != len(v):
            raise ValueError("pos4 and vel4 lengths differ")
        w = None if omega4 is None else _f32(omega4)
        self._call("sd_engine_add_spheres", len(p), p.ctypes.data, v.ctypes.data,
                   None if w is None else w.ctypes.data)
        self._n += len(p)

    def remove_spheres(self, ids) -> None:
        """Removes free spheres by id (before or after prepare); the others
        keep their order and take ids 0..n-1 in it."""
        i = np.ascontiguousarray(ids, np.uint32)
        self._call("sd_engine_remove_spheres", len(i), i.ctypes.data)
        self._n -= len(i)

    def add(self, grid_resolution: int, size: float, diameter: float, mass: float, position, velocity) -> None:
        """DEMEngine::add(DEMParticle(...)): one sphere, or a rigid cube clump
        of floor(size/diameter)^2 spheres when grid_resolution > 1."""
        p = (C.c_float * 3)(*position)
        v = (C.c_float * 3)(*velocity)
        self._call("sd_engine_add_particle", grid_resolution, size, diameter, mass, p, v)
        self._n = int(self.stats()["n_spheres"])

    def add_scene(self, pos4, vel4, lo, hi, cell: float = 0.0, omega4=None) -> None:
        """One scene of a batch: spheres in their own walled box [lo, hi]."""
        p = _f32(pos4)
        v = _f32(vel4)
        w = None if omega4 is None else _f32(omega4)
        lo3 = (C.c_float * 3)(*lo)
        hi3 = (C.c_float * 3)(*hi)
        self._call("sd_engine_add_scene", len(p), p.ctypes.data, v.ctypes.data, None if w is None else w.ctypes.data,
                   lo3, hi3, cell)
        self._n += len(p)
        self.n_scenes = getattr(self, "n_scenes", 0) + 1

    def add_mesh(self, tris, centre, axis=(0.0, 0.0, 1.0), omega: float = 0.0, patch=None) -> None:
        """A rigid triangle mesh (tris: (n, 3, 3) world vertices at time 0)
        rotating at omega about the line through centre along axis."""
        t = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
        pa = None if patch is None else np.ascontiguousarray(patch, np.int32)
        c = (C.c_float * 3)(*centre)
        a = (C.c_float * 3)(*axis)
        self._call("sd_engine_add_mesh", len(t), t.ctypes.data, None if pa is None else pa.ctypes.data, c, a, omega)

    def add_mesh_stl(self, path, position=None, quaternion=None, centre=None, axis=(0.0, 0.0, 1.0),
                     omega: float = 0.0, patch_angle: float = 30.0) -> None:
        """DEMMesh(filename, position, quaternion): an STL file's triangles
        placed at R(quaternion) v + position (quaternion (s, x, y, z)), grouped
        into smooth patches (crease angle patch_angle degrees), static or
        rotating at omega about the line through centre along axis."""
        def arr(v, n):
            return None if v is None else (C.c_float * n)(*v)
        self._call("sd_engine_add_mesh_stl", str(path).encode(), arr(position, 3), arr(quaternion, 4), arr(centre, 3),
                   arr(axis, 3), omega, patch_angle)

    def mesh(self):
        """The engine's mesh as it steps it: (triangles in the mesh frame,
        (n, 3, 3); patch ids; centre) -- world at time 0 = frame + centre."""
        n = C.c_uint64()
        self._call("sd_engine_get_mesh", 0, None, None, None, C.byref(n))
        t = np.empty((n.value, 3, 3), np.float32)
        pa = np.empty(n.value, np.int32)
        c = (C.c_float * 3)()
        self._call("sd_engine_get_mesh", n.value, t.ctypes.data, pa.ctypes.data, c, C.byref(n))
        return t, pa, tuple(c)

    def write_snapshot(self, path, fmt: str = "vtk", contacts: bool = False, mesh: bool = False) -> None:
        """Writes the state to a CSV or legacy-VTK file (sd_engine_write_snapshot)."""
        kinds = {"csv": _abi.SD_SNAPSHOT_CSV, "vtk": _abi.SD_SNAPSHOT_VTK}
        if fmt not in kinds:
            raise ValueError("fmt must be 'csv' or 'vtk'")
        flags = (_abi.SD_SNAPSHOT_CONTACTS if contacts else 0) | (_abi.SD_SNAPSHOT_MESH if mesh else 0)
        self._call("sd_engine_write_snapshot", str(path).encode(), kinds[fmt], flags)

    def mesh_state(self) -> np.ndarray:
        out = np.empty(24, np.float32)
        self._call("sd_engine_get_mesh_state", out.ctypes.data)
        return out

    def add_clump(self, rel4, mass: float, com, velocity=(0.0, 0.0, 0.0), omega=(0.0, 0.0, 0.0)) -> None:
        """One rigid body made of spheres (rel4 rows: body-frame offset from
        the centre of mass, radius); the body's inertia is that of its
        spheres as solid balls of mass/n each."""
        r = _f32(rel4)
        c = (C.c_float * 3)(*com)
        v = (C.c_float * 3)(*velocity)
        w = (C.c_float * 3)(*omega)
        self._call("sd_engine_add_clump", len(r), r.ctypes.data, mass, c, v, w)
        self._n += len(r)

    @property
    def n_bodies(self) -> int:
        return int(self.stats()["n_bodies"])

    # -- convex hulls
    def add_hull(self, points, mass: float, position, quat=None, velocity=(0.0, 0.0, 0.0),
                 omega=(0.0, 0.0, 0.0)) -> None:
        """One convex hull of `points` (n x 3, local frame) at `position`
        with orientation `quat` (s, x, y, z)."""
        pts = np.zeros((len(points), 4), np.float32)
        pts[:, :3] = np.asarray(points, np.float32)
        p = (C.c_float * 3)(*position)
        q = None if quat is None else (C.c_float * 4)(*quat)
        v = (C.c_float * 3)(*velocity)
        w = (C.c_float * 3)(*omega)
        self._call("sd_engine_add_hull", len(pts), pts.ctypes.data, mass, p, q, v, w)

    def hull_shapes(self):
        """(vstart, vcount, principal-frame vertices float4)."""
        nb = self.n_bodies
        nv = C.c_uint64()
        self._call("sd_engine_get_hull_shapes", None, None, None, 0, C.byref(nv))
        vs = np.empty(nb, np.uint32)
        vc = np.empty(nb, np.uint32)
        verts = np.empty((max(nv.value, 1), 4), np.float32)
        self._call("sd_engine_get_hull_shapes", vs.ctypes.data, vc.ctypes.data, verts.ctypes.data, nv.value,
                   C.byref(nv))
        return vs, vc, verts[: nv.value]

    def set_gjk_seed(self, mode: int) -> None:
        self._call("sd_engine_set_gjk_seed", mode)

    def set_gjk_training(self, every: int, iters: int, lr: float = 1e-3) -> None:
        """Online training of the warm-start network (sd_engine_set_gjk_training)."""
        self._call("sd_engine_set_gjk_training", every, iters, lr)

    def hull_entries(self) -> dict:
        """The last step's candidate entries (CSR) with status, iterations,
        final directions, seeds and network inputs."""
        nb = self.n_bodies
        m = C.c_uint64()
        off = np.empty(nb + 1, np.uint32)
        self._call("sd_engine_hull_entries", off.ctypes.data, None, None, None, None, None, 0, C.byref(m))
        n = m.value
        part = np.empty(max(n, 1), np.uint32)
        info = np.empty(max(n, 1), np.uint32)
        d4 = np.empty((max(n, 1), 4), np.float32)
        s4 = np.empty((max(n, 1), 4), np.float32)
        f16 = np.empty((max(n, 1), 16), np.float32)
        self._call("sd_engine_hull_entries", off.ctypes.data, part.ctypes.data, info.ctypes.data, d4.ctypes.data,
                   s4.ctypes.data, f16.ctypes.data, n, C.byref(m))
        return {"off": off, "partners": part[:n], "status": (info[:n] & 0xFF).astype(np.int32),
                "iters": ((info[:n] >> 8) & 0xFF).astype(np.int32), "epa_iters": ((info[:n] >> 16) & 0xFF).astype(np.int32),
                "dir": d4[:n], "seeds": s4[:n], "feat": f16[:n]}

    # -- GJK warm-start network (hull scenes)
    def mlp_params(self) -> np.ndarray:
        out = np.empty(6288, np.float32)
        self._call("sd_engine_mlp_params", out.ctypes.data, 6288, 0)
        return out

    def set_mlp_params(self, params) -> None:
        p = np.ascontiguousarray(params, np.float32)
        self._call("sd_engine_mlp_params", p.ctypes.data, p.size, 1)

    def mlp_forward(self, feat16):
        """feat16: CUDA float32 tensor (n, 16) -> (n, 4) tensor (y0, y1, y2, 0)."""
        import torch
        out = torch.empty((feat16.shape[0], 4), dtype=torch.float32, device=feat16.device)
        self._call("sd_engine_mlp_forward", feat16.data_ptr(), out.data_ptr(), feat16.shape[0])
        return out

    def mlp_train(self, feat16, tgt4, iters: int, lr: float = 1e-3) -> np.ndarray:
        """Full-batch Adam steps on CUDA tensors; returns the last gradient."""
        g = np.empty(6288, np.float32)
        self._call("sd_engine_mlp_train", feat16.data_ptr(), tgt4.data_ptr(), feat16.shape[0], iters, lr,
                   g.ctypes.data)
        return g

    def bodies(self, field: int) -> np.ndarray:
        """Rigid-body field (SD_BODY_*), one float4 row per body (3 rows per
        body for SD_BODY_INV_INERTIA)."""
        nb = self.n_bodies
        rows = 3 * nb if field == _abi.SD_BODY_INV_INERTIA else nb
        out = np.empty((rows, 4), dtype=np.float32)
        self._call("sd_engine_get_bodies", field, out.ctypes.data, out.nbytes)
        return out

    def load_scene_json(self, path: str) -> None:
        self._call("sd_engine_load_scene_json", str(path).encode())
        st = self.stats()
        self._n = int(st["n_spheres"])

    def prepare(self) -> None:
        self._call("sd_engine_prepare")

    # reference names: prep() builds host arrays, transfer() uploads
    def prep(self) -> None:
        pass

    def transfer(self) -> None:
        self.prepare()

    # -- stepping
    def step(self, dt: float, n_steps: int = 1) -> None:
        self._call("sd_engine_step", dt, n_steps)

    def update(self, dt: float) -> None:
        self._call("sd_engine_update", dt)

    def sync(self) -> None:
        self._call("sd_engine_sync")

    # -- state
    @property
    def n(self) -> int:
        return self._n

    def get(self, field: int) -> np.ndarray:
        out = np.empty((self._n, 4), dtype=np.float32)
        self._call("sd_engine_get_state", field, out.ctypes.data, out.nbytes)
        return out

    def set(self, field: int, arr) -> None:
        a = _f32(arr)
        self._call("sd_engine_set_state", field, a.ctypes.data, a.nbytes)

    def positions(self) -> np.ndarray:
        return self.get(_abi.SD_FIELD_POSITION)

    def velocities(self) -> np.ndarray:
        return self.get(_abi.SD_FIELD_VELOCITY)

    def omegas(self) -> np.ndarray:
        return self.get(_abi.SD_FIELD_OMEGA)

    def forces(self) -> np.ndarray:
        return self.get(_abi.SD_FIELD_FORCE)

    def torques(self) -> np.ndarray:
        return self.get(_abi.SD_FIELD_TORQUE)

    def device_ptr(self, field: int) -> int:
        p = C.c_void_p()
        self._call("sd_engine_device_ptr", field, C.byref(p))
        return p.value

    def stream(self) -> int:
        p = C.c_void_p()
        self._call("sd_engine_stream", C.byref(p))
        return p.value or 0

    def pairs(self, cap: int | None = None) -> np.ndarray:
        n = C.c_uint64()
        cap = self.config.pair_capacity if cap is None else cap
        out = np.empty(max(cap, 1), dtype=np.uint64)
        self._call("sd_engine_get_pairs", out.ctypes.data, cap, C.byref(n))
        return out[: n.value].copy()

    def stats(self) -> dict:
        s = _abi.SdStats()
        self._call("sd_engine_stats", C.byref(s))
        return {
            "n_spheres": s.n_spheres, "steps": s.steps, "contacts": s.contacts,
            "kinetic_energy": s.kinetic_energy, "momentum": tuple(s.momentum),
            "device_errors": s.device_errors, "n_cells": s.n_cells, "n_bodies": s.n_bodies,
            "gjk_pairs": s.gjk_pairs, "gjk_iters": s.gjk_iters, "epa_iters": s.epa_iters,
            "moved_keys": s.moved_keys, "step_kernels": s.step_kernels,
            "list_builds": s.list_builds, "listed_steps": s.listed_steps,
        }

    def params(self) -> dict:
        p = _abi.SdParams()
        self._call("sd_engine_params", C.byref(p))
        return {"lo": tuple(p.lo), "hi": tuple(p.hi), "cell": p.cell, "dims": (p.nx, p.ny, p.nz),
                "kn": p.kn, "damp": p.damp, "mu": p.mu, "gravity": tuple(p.gravity), "dt": p.dt,
                "walls": p.walls, "rmax": p.rmax, "cell_z": p.cell_z, "z_div": p.z_div}

    def save_checkpoint(self, path: str) -> None:
        self._call("sd_engine_save_checkpoint", str(path).encode())

    def load_checkpoint(self, path: str) -> None:
        self._call("sd_engine_load_checkpoint", str(path).encode())
        self._n = int(self.stats()["n_spheres"])


def scene_lattice(nx, ny, nz, spacing, jitter, origin, radius, mass, vmax, seed):
    """Seeded jittered cubic lattice (sd_scene_lattice)."""
    n = nx * ny * nz
    pos = np.empty((n, 4), np.float32)
    vel = np.empty((n, 4), np.float32)
    o = (C.c_float * 3)(*origin)
    call("sd_scene_lattice", nx, ny, nz, spacing, jitter, o, radius, mass, vmax, seed,
         pos.ctypes.data, vel.ctypes.data)
    return pos, vel


def scene_rsa(n, lo, hi, r_median, r_sigma, r_min, r_max, density, vmax, seed, max_attempts=50_000_000):
    """Seeded random-sequential-addition packing (sd_scene_rsa)."""
    pos = np.empty((n, 4), np.float32)
    vel = np.empty((n, 4), np.float32)
    phi = C.c_double()
    call("sd_scene_rsa", n, (C.c_float * 3)(*lo), (C.c_float * 3)(*hi), r_median, r_sigma, r_min, r_max,
         density, vmax, seed, max_attempts, pos.ctypes.data, vel.ctypes.data, C.byref(phi))
    return pos, vel, phi.value


class SpatialPartition:
    """Reference operator class over CUDA tensors (torch), bit-exact broad phase."""

    @staticmethod
    def _stream(stream):
        if stream is None:
            import torch
            return C.c_void_p(torch.cuda.current_stream().cuda_stream)
        return C.c_void_p(stream)

    @staticmethod
    def construct_collision_list(n, cell_dim, cells, spheres, sizes, pos4, count, stream=None):
        """constructCollisionList: 9n (cell, sphere) entries + valid count."""
        call("sd_hash_construct_collision_list", n, cell_dim, cells.data_ptr(), spheres.data_ptr(),
             sizes.data_ptr(), pos4.data_ptr(), count.data_ptr(), SpatialPartition._stream(stream))

    @staticmethod
    def sort_scratch_bytes(n, key_bits=32) -> int:
        b = C.c_uint64()
        call("sd_sort_scratch_bytes", n, key_bits, C.byref(b))
        return b.value

    @staticmethod
    def sort_collision_list(cells, spheres, cells_tmp, spheres_tmp, n, scratch, stream=None):
        """sortCollisionList: stable sort of the first n entries by cell word."""
        call("sd_hash_sort_collision_list", cells.data_ptr(), spheres.data_ptr(), cells_tmp.data_ptr(),
             spheres_tmp.data_ptr(), n, scratch.data_ptr(), scratch.numel() * scratch.element_size(),
             SpatialPartition._stream(stream))

    @staticmethod
    def sort_pairs(keys, vals, keys_tmp, vals_tmp, n, key_bits, scratch, stream=None):
        call("sd_sort_pairs", keys.data_ptr(), vals.data_ptr(), keys_tmp.data_ptr(), vals_tmp.data_ptr(), n,
             key_bits, scratch.data_ptr(), scratch.numel() * scratch.element_size(),
             SpatialPartition._stream(stream))

    @staticmethod
    def sort_status(scratch, stream=None) -> int:
        v = C.c_uint32()
        call("sd_sort_status", scratch.data_ptr(), SpatialPartition._stream(stream), C.byref(v))
        return v.value

    @staticmethod
    def pairs_scratch_bytes(n_entries) -> int:
        b = C.c_uint64()
        call("sd_hash_pairs_scratch_bytes", n_entries, C.byref(b))
        return b.value

    @staticmethod
    def candidate_pairs(cells, spheres, count, n_entries, body_of, pair_a, pair_b, cap, npairs, scratch,
                        stream=None):
        """Candidate pairs of tranverseAndResolveCollisionList's run traversal."""
        call("sd_hash_candidate_pairs", cells.data_ptr(), spheres.data_ptr(), count.data_ptr(), n_entries,
             None if body_of is None else body_of.data_ptr(), pair_a.data_ptr(), pair_b.data_ptr(), cap,
             npairs.data_ptr(), scratch.data_ptr(), scratch.numel() * scratch.element_size(),
             SpatialPartition._stream(stream))


class BoundingVolumes:
    """LBVH broad phase over boxes (sandbox/testLBVH.cu as raw device
    operators) on CUDA tensors: lo/hi are (n, 4) float32 (x, y, z, -)."""

    @staticmethod
    def scratch_bytes(n: int, pair_cap: int) -> int:
        b = C.c_uint64()
        call("sd_lbvh_scratch_bytes", n, pair_cap, C.byref(b))
        return b.value

    @staticmethod
    def pairs(lo, hi, cap: int, stream=None):
        """Ascending unique pairs (i < j) of overlapping boxes as an int64
        tensor of (i << 32 | j), and the device error bits."""
        import torch
        n = lo.shape[0]
        scratch = torch.empty(BoundingVolumes.scratch_bytes(n, cap), dtype=torch.uint8, device=lo.device)
        out = torch.empty(max(cap, 1), dtype=torch.int64, device=lo.device)
        cnt = torch.zeros(2, dtype=torch.int32, device=lo.device)
        call("sd_lbvh_pairs", n, lo.data_ptr(), hi.data_ptr(), out.data_ptr(), cap, cnt.data_ptr(),
             scratch.data_ptr(), scratch.numel(), SpatialPartition._stream(stream))
        c = cnt.cpu().numpy().view(np.uint32)
        return out[: min(int(c[0]), cap)], int(c[0]), int(c[1])

    @staticmethod
    def morton(lo, hi, stream=None):
        import torch
        n = lo.shape[0]
        scratch = torch.empty(BoundingVolumes.scratch_bytes(n, 0), dtype=torch.uint8, device=lo.device)
        codes = torch.empty(max(n, 1), dtype=torch.int32, device=lo.device)
        call("sd_lbvh_morton", n, lo.data_ptr(), hi.data_ptr(), codes.data_ptr(), scratch.data_ptr(),
             scratch.numel(), SpatialPartition._stream(stream))
        return codes[:n]


def add_hull_scene(eng: DEMEngine, points, pos, quat, vel, mass, omega=None) -> None:
    """Adds scenes.hull_box's hulls in order."""
    for i in range(len(points)):
        eng.add_hull(points[i], float(mass[i]), tuple(pos[i]), tuple(quat[i]), tuple(vel[i]),
                     (0.0, 0.0, 0.0) if omega is None else tuple(omega[i]))


class SweepAndPrune:
    """SAPCollision (src/engine/cuda/collisions/SAP/sap_detection.cu) as raw
    device operators on CUDA tensors."""

    @staticmethod
    def scratch_bytes(n: int, pair_cap: int = 0) -> int:
        b = C.c_uint64()
        call("sd_sap_scratch_bytes", n, pair_cap, C.byref(b))
        return b.value

    @staticmethod
    def pairs(lo, hi, cap: int, stream=None):
        """Exact pair set: (int64 tensor of (i << 32 | j) ascending, count, device error bits)."""
        import torch
        n = lo.shape[0]
        scratch = torch.empty(SweepAndPrune.scratch_bytes(n, cap), dtype=torch.uint8, device=lo.device)
        out = torch.empty(max(cap, 1), dtype=torch.int64, device=lo.device)
        cnt = torch.zeros(2, dtype=torch.int32, device=lo.device)
        call("sd_sap_pairs", n, lo.data_ptr(), hi.data_ptr(), out.data_ptr(), cap, cnt.data_ptr(), scratch.data_ptr(),
             scratch.numel(), SpatialPartition._stream(stream))
        c = cnt.cpu().numpy().view(np.uint32)
        return out[: min(int(c[0]), cap)], int(c[0]), int(c[1])

    @staticmethod
    def sweep(upperx, lowerx_sorted, uppery, lowery, idx_sorted, stream=None):
        """sweepAndPruneCUDA rows (n, 16) int32 on given sorted inputs."""
        import torch
        n = upperx.shape[0]
        rows = torch.empty((max(n, 1), 16), dtype=torch.int32, device=upperx.device)
        call("sd_sap_sweep", n, upperx.data_ptr(), lowerx_sorted.data_ptr(), uppery.data_ptr(), lowery.data_ptr(),
             idx_sorted.data_ptr(), rows.data_ptr(), SpatialPartition._stream(stream))
        return rows[:n]

    @staticmethod
    def process_collisions(pos4, radius=None, stream=None):
        """SAPCollision::processCollisions: rows (n, 16) int32 per sorted position."""
        import torch
        n = pos4.shape[0]
        scratch = torch.empty(SweepAndPrune.scratch_bytes(n, 0), dtype=torch.uint8, device=pos4.device)
        rows = torch.empty((max(n, 1), 16), dtype=torch.int32, device=pos4.device)
        call("sd_sap_process_collisions", n, pos4.data_ptr(), None if radius is None else radius.data_ptr(),
             rows.data_ptr(), scratch.data_ptr(), scratch.numel(), SpatialPartition._stream(stream))
        return rows[:n]
