"""ctypes front end of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU legs, as the checker or as the timed CPU restatement.  The
product library never loads it.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_lib = None


class Params(C.Structure):
    """sdo_params (oracle/sd_oracle.h)."""
    _fields_ = [
        ("lo", C.c_float * 3), ("hi", C.c_float * 3), ("cell", C.c_float),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("kn", C.c_float), ("damp", C.c_float), ("mu", C.c_float),
        ("g", C.c_float * 3), ("dt", C.c_float), ("walls", C.c_int32),
        ("cell_z", C.c_float),
    ]


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        from . import build as _build  # noqa: F401  (package-relative when imported as oracle.oracle)
        path = HERE / "liboracle.so"
        if not path.exists():
            _build.build()
        l = C.CDLL(str(path))
        P = C.c_void_p
        sig = {
            "sdo_ref_hash_build": (C.c_uint32, [C.c_uint32, C.c_float, P, P, P, P]),
            "sdo_radix_sort_pairs": (None, [P, P, C.c_uint32, C.c_int, P, P]),
            "sdo_ref_candidate_pairs": (C.c_uint64, [P, P, C.c_uint32, P, P, P, C.c_uint64]),
            "sdo_ref_resolve_forces": (None, [P, P, C.c_uint32, P, P, P, P]),
            "sdo_ref_update_spheres": (None, [C.c_int, P, P, P, P, P, P, P, P, P]),
            "sdo_ref_body_forces": (None, [C.c_int, P, P, P, P, P, P, P]),
            "sdo_ref_advect": (None, [C.c_int, C.c_float, P, P, P, P, P, P, P, P, P, P]),
            "sdo_cell_key": (C.c_uint32, [P, C.c_float, C.c_float, C.c_float]),
            "sdo_cell_keys": (None, [P, C.c_uint32, P, P]),
            "sdo_sort_reorder": (None, [P, C.c_uint32, P, P, P, P, P, P, P, P, P]),
            "sdo_contact_integrate": (C.c_uint64, [P, C.c_uint32, P, P, P, P, P, P, P, P, P, P]),
            "sdo_contact_integrate_f64": (C.c_uint64, [P, C.c_uint32, P, P, P, P, P, P, P, P, P, P]),
            "sdo_contact_pairs": (C.c_uint64, [P, C.c_uint32, P, P, P, P, C.c_uint64]),
            "sdo_run": (C.c_int, [P, C.c_uint32, P, P, P, C.c_int, C.c_int]),
            "sdo_run_f64": (C.c_int, [P, C.c_uint32, P, P, P, P, C.c_int, P]),
            "sdo_contact_integrate_bodies": (C.c_uint64, [P, C.c_uint32] + [P] * 13),
            "sdo_slot_of": (None, [C.c_uint32, P, P]),
            "sdo_body_step": (None, [P, C.c_uint32] + [P] * 18),
            "sdo_run_bodies": (C.c_int, [P, C.c_uint32, P, P, P, C.c_int, C.c_uint32] + [P] * 10),
            "sdo_morton_ref": (None, [C.c_uint32, P, P, P, P, P]),
            "sdo_aabb_pairs": (C.c_uint64, [C.c_uint32, P, P, P, C.c_uint64]),
            "sdo_hull_aabbs": (None, [C.c_uint32, P, P, P, P, P, P, P, P]),
            "sdo_gjk_epa": (None, [P, P, P, P, P, P, C.c_uint32, C.c_uint32, P, P, P]),
            "sdo_hull_partners": (C.c_int64, [C.c_uint32, P, P, P, P, C.c_uint64]),
            "sdo_hull_step": (None, [P, C.c_uint32] + [P] * 17),
            "sdo_sap_sweep_ref": (None, [C.c_uint32, P, P, P, P, P, P]),
            "sdo_sap_process": (None, [C.c_uint32, P, P, P]),
            "sdo_run_full": (C.c_int, [P, C.c_uint32, P, P, P, C.c_int, C.c_uint32] + [P] * 11),
            "sdo_mesh_advance": (None, [P, C.c_int]),
            "sdo_scene_lattice": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_float, P, C.c_float,
                                            C.c_float, C.c_float, C.c_uint64, P, P]),
            "sdo_scene_rsa": (C.c_int, [C.c_uint64, P, P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                        C.c_float, C.c_uint64, C.c_uint64, P, P, C.POINTER(C.c_double)]),
            "sdo_num_threads": (C.c_int, []),
            "sdo_set_num_threads": (None, [C.c_int]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


# ------------------------------------------------------------ scene inputs
def scene_lattice(nx, ny, nz, spacing, jitter, origin, radius, mass, vmax, seed):
    """The library's seeded lattice builder, compiled into the oracle
    (stardust_gb300/csrc/sd_scenes.cu): same arguments and output."""
    n = nx * ny * nz
    pos = np.empty((n, 4), np.float32)
    vel = np.empty((n, 4), np.float32)
    rc = lib().sdo_scene_lattice(nx, ny, nz, spacing, jitter, (C.c_float * 3)(*origin), radius, mass, vmax, seed,
                                 _p(pos), _p(vel))
    if rc != 0:
        raise RuntimeError(f"scene_lattice failed ({rc})")
    return pos, vel


def scene_rsa(n, lo, hi, r_median, r_sigma, r_min, r_max, density, vmax, seed, max_attempts=50_000_000):
    """The library's seeded RSA packing, compiled into the oracle."""
    pos = np.empty((n, 4), np.float32)
    vel = np.empty((n, 4), np.float32)
    phi = C.c_double()
    rc = lib().sdo_scene_rsa(n, (C.c_float * 3)(*lo), (C.c_float * 3)(*hi), r_median, r_sigma, r_min, r_max,
                             density, vmax, seed, max_attempts, _p(pos), _p(vel), C.byref(phi))
    if rc != 0:
        raise RuntimeError(f"scene_rsa failed ({rc})")
    return pos, vel, phi.value


# ---------------------------------------------------------------- ref_compat
def ref_hash_build(pos4: np.ndarray, sizes: np.ndarray, cell_dim: float):
    n = len(pos4)
    pos4 = np.ascontiguousarray(pos4, np.float32)
    sizes = np.ascontiguousarray(sizes, np.float32)
    cells = np.empty(9 * n, np.uint32)
    spheres = np.empty(9 * n, np.uint32)
    count = lib().sdo_ref_hash_build(n, cell_dim, _p(pos4), _p(sizes), _p(cells), _p(spheres))
    return cells, spheres, int(count)


def radix_sort_pairs(keys: np.ndarray, vals: np.ndarray, nbits: int = 32):
    k = np.array(keys, np.uint32, copy=True)
    v = np.array(vals, np.uint32, copy=True)
    tk = np.empty_like(k)
    tv = np.empty_like(v)
    lib().sdo_radix_sort_pairs(_p(k), _p(v), len(k), nbits, _p(tk), _p(tv))
    return k, v


def ref_candidate_pairs(cells, spheres, count, body_of=None):
    cells = np.ascontiguousarray(cells, np.uint32)
    spheres = np.ascontiguousarray(spheres, np.uint32)
    bo = None if body_of is None else np.ascontiguousarray(body_of, np.int32)
    n = lib().sdo_ref_candidate_pairs(_p(cells), _p(spheres), count, _p(bo), None, None, 0)
    a = np.empty(max(n, 1), np.uint32)
    b = np.empty(max(n, 1), np.uint32)
    lib().sdo_ref_candidate_pairs(_p(cells), _p(spheres), count, _p(bo), _p(a), _p(b), n)
    return a[:n], b[:n]


def ref_resolve_forces(cells, spheres, count, pos4, vel4, body_of=None):
    pos4 = np.ascontiguousarray(pos4, np.float32)
    vel4 = np.ascontiguousarray(vel4, np.float32)
    f = np.zeros_like(pos4)
    bo = None if body_of is None else np.ascontiguousarray(body_of, np.int32)
    lib().sdo_ref_resolve_forces(_p(np.ascontiguousarray(cells, np.uint32)),
                                 _p(np.ascontiguousarray(spheres, np.uint32)), count, _p(bo), _p(pos4),
                                 _p(vel4), _p(f))
    return f


# ------------------------------------------------------------------- physics
def _key_bits(ncells: int) -> int:
    """Bits of a cell key over ncells cells (at least 1, at most 32)."""
    b = 1
    while b < 32 and (1 << b) < ncells:
        b += 1
    return b


def _sort_passes(bits: int) -> int:
    """Digit passes of the step's radix sort for keys of `bits` bits: 9-bit
    digits, except that 19- and 20-bit keys take two 10-bit passes."""
    bits = min(max(bits, 1), 32)
    return 2 if bits in (19, 20) else (bits + 8) // 9


def auto_z_div(ncells: int) -> int:
    """The automatic z split of a single scene's grid: the larger of 4 and 2
    whose finer grid keeps keys within 20 bits and sorts in as many passes
    as the plain grid, else 1."""
    p0 = _sort_passes(_key_bits(ncells))
    for zd in (4, 2):
        bits = _key_bits(ncells * zd)
        if bits <= 20 and _sort_passes(bits) == p0:
            return zd
    return 1


def derive_params(cfg, radii, dt: float, z_div: int | None = None) -> Params:
    """The step parameters of a single scene, derived here from the scene
    config and the sphere radii (not read back from the engine).

    cfg: an object with box_lo, box_hi, domain, cell, kn, restitution, mu,
    gravity, walls (the engine config's fields).  Box: box_lo..box_hi, or
    0..domain on every axis when box_hi is all zero.  Cell edge: cfg.cell,
    or 2 x the largest radius when it is 0.  Cells per axis:
    ceil(edge / cell * (1 - 1e-6)) in double (at least 1), so a float cell
    that divides the edge gives the exact count.  z split: z_div when given
    (1 when the finer grid would exceed 2^30 cells), else auto_z_div.
    cell_z = cell / z_div in float.  Normal damping: damp_from(kn, e)."""
    f32 = np.float32
    given = any(float(v) != 0.0 for v in cfg.box_hi)
    lo = [f32(cfg.box_lo[a]) if given else f32(0.0) for a in range(3)]
    hi = [f32(cfg.box_hi[a]) if given else f32(cfg.domain) for a in range(3)]
    r = np.asarray(radii, np.float32)
    rmax = f32(r.max()) if r.size else f32(0.0)
    cell = f32(cfg.cell) if cfg.cell > 0 else f32(2.0) * rmax
    if not cell > 0:
        cell = hi[0] - lo[0]
    dims = [max(1, int(math.ceil((float(hi[a]) - float(lo[a])) / float(cell) * (1.0 - 1e-6)))) for a in range(3)]
    ncells = dims[0] * dims[1] * dims[2]
    if z_div is not None and z_div > 0:
        zd = z_div if ncells * z_div <= (1 << 30) else 1
    else:
        zd = auto_z_div(ncells)
    p = Params()
    for a in range(3):
        p.lo[a] = lo[a]
        p.hi[a] = hi[a]
        p.g[a] = cfg.gravity[a]
    p.cell = cell
    p.nx, p.ny, p.nz = dims[0], dims[1], dims[2] * zd
    p.cell_z = f32(cell / f32(zd))
    p.kn = cfg.kn
    p.damp = damp_from(cfg.kn, cfg.restitution)
    p.mu = cfg.mu
    p.dt = dt
    p.walls = cfg.walls
    return p


def params_checked(cfg, radii, dt: float, engine_params: dict, z_div: int | None = None) -> Params:
    """derive_params, then a check that the engine derived the same grid and
    contact-law constants (engine_params = its sd_engine_params): box, cell,
    cells per axis, cell_z, kn, damp, mu, gravity, walls, bit for bit.
    Raises AssertionError naming every field that differs."""
    p = derive_params(cfg, radii, dt, z_div)
    f = lambda x: np.float32(x).view(np.uint32)  # noqa: E731
    ep = engine_params
    bad = []
    for a in range(3):
        if f(p.lo[a]) != f(ep["lo"][a]) or f(p.hi[a]) != f(ep["hi"][a]):
            bad.append(f"box axis {a}: oracle {p.lo[a]}..{p.hi[a]}, engine {ep['lo'][a]}..{ep['hi'][a]}")
        if f(p.g[a]) != f(ep["gravity"][a]):
            bad.append(f"gravity {a}")
    if f(p.cell) != f(ep["cell"]):
        bad.append(f"cell: oracle {p.cell}, engine {ep['cell']}")
    if (p.nx, p.ny, p.nz) != tuple(ep["dims"]):
        bad.append(f"dims: oracle {(p.nx, p.ny, p.nz)}, engine {tuple(ep['dims'])}")
    if f(p.cell_z) != f(ep["cell_z"]):
        bad.append(f"cell_z: oracle {p.cell_z}, engine {ep['cell_z']}")
    for k in ("kn", "damp", "mu"):
        if f(getattr(p, k)) != f(ep[k]):
            bad.append(f"{k}: oracle {getattr(p, k)}, engine {ep[k]}")
    if p.walls != ep["walls"]:
        bad.append("walls")
    if bad:
        raise AssertionError("engine parameters differ from the oracle's: " + "; ".join(bad))
    return p


def make_params(lo, hi, cell, kn, damp, mu, g, dt, walls) -> Params:
    p = Params()
    for a in range(3):
        p.lo[a] = lo[a]
        p.hi[a] = hi[a]
        p.g[a] = g[a]
    p.cell = cell
    dims = [max(1, int(np.ceil((np.float64(np.float32(hi[a])) - np.float64(np.float32(lo[a])))
                               / np.float64(np.float32(cell))))) for a in range(3)]
    p.nx, p.ny, p.nz = dims
    p.kn = kn
    p.damp = damp
    p.mu = mu
    p.dt = dt
    p.walls = walls
    return p


def damp_from(kn: float, e: float) -> float:
    le = np.log(np.float64(np.float32(e)))
    beta = -le / np.sqrt(np.pi ** 2 + le * le)
    return float(np.float32(2.0 * beta * np.sqrt(np.float64(np.float32(kn)))))


def ncells(p: Params) -> int:
    return p.nx * p.ny * p.nz


def with_ids(omg: np.ndarray, ids: np.ndarray) -> np.ndarray:
    o = np.array(omg, np.float32, copy=True)
    o.view(np.uint32)[:, 3] = np.asarray(ids, np.uint32) & 0x7FFFFFFF
    return o


def ids_of(omg: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(omg, np.float32).view(np.uint32)[:, 3] & 0x7FFFFFFF


def cell_keys(p: Params, pos4: np.ndarray) -> np.ndarray:
    pos4 = np.ascontiguousarray(pos4, np.float32)
    keys = np.empty(len(pos4), np.uint32)
    lib().sdo_cell_keys(C.byref(p), len(pos4), _p(pos4), _p(keys))
    return keys


def sort_reorder(p: Params, pos_n, vel_n, omg_n, keys):
    n = len(pos_n)
    pos = np.empty((n, 4), np.float32)
    vel = np.empty((n, 4), np.float32)
    omg = np.empty((n, 4), np.float32)
    ks = np.empty(n, np.uint32)
    cs = np.empty(ncells(p) + 1, np.uint32)
    lib().sdo_sort_reorder(C.byref(p), n, _p(np.ascontiguousarray(pos_n, np.float32)),
                           _p(np.ascontiguousarray(vel_n, np.float32)), _p(np.ascontiguousarray(omg_n, np.float32)),
                           _p(np.ascontiguousarray(keys, np.uint32)), _p(ks), _p(pos), _p(vel), _p(omg), _p(cs))
    return pos, vel, omg, ks, cs


def prepare(p: Params, pos4, vel4, omg4):
    """Initial cell sort of a state given in insertion order (ids in omg.w)."""
    pos4 = np.ascontiguousarray(pos4, np.float32)
    return sort_reorder(p, pos4, vel4, omg4, cell_keys(p, pos4))


def contact_integrate(p: Params, pos, vel, omg, cs, record=True, f64=False):
    n = len(pos)
    dt = np.float64 if f64 else np.float32
    pos_n = np.empty((n, 4), dt)
    vel_n = np.empty((n, 4), dt)
    omg_n = np.empty((n, 4), dt)
    keys = np.empty(n, np.uint32)
    f = np.empty((n, 4), dt) if record else None
    t = np.empty((n, 4), dt) if record else None
    fn = lib().sdo_contact_integrate_f64 if f64 else lib().sdo_contact_integrate
    c = fn(C.byref(p), n, _p(np.ascontiguousarray(pos, dt)), _p(np.ascontiguousarray(vel, dt)),
           _p(np.ascontiguousarray(omg, dt)), _p(np.ascontiguousarray(cs, np.uint32)), _p(pos_n), _p(vel_n),
           _p(omg_n), _p(keys), _p(f), _p(t))
    return pos_n, vel_n, omg_n, keys, f, t, int(c)


def contact_pairs(p: Params, pos, omg, cs, cap=1 << 22):
    out = np.empty(cap, np.uint64)
    n = lib().sdo_contact_pairs(C.byref(p), len(pos), _p(np.ascontiguousarray(pos, np.float32)),
                                _p(np.ascontiguousarray(omg, np.float32)), _p(np.ascontiguousarray(cs, np.uint32)),
                                _p(out), cap)
    if n > cap:
        raise RuntimeError("pair capacity")
    return out[:n].copy()


def run(p: Params, pos, vel, omg, steps: int, prepare_first: bool = True):
    """sdo_run: returns the cell-sorted state after `steps` steps."""
    pos = np.array(pos, np.float32, copy=True)
    vel = np.array(vel, np.float32, copy=True)
    omg = np.array(omg, np.float32, copy=True)
    rc = lib().sdo_run(C.byref(p), len(pos), _p(pos), _p(vel), _p(omg), steps, 1 if prepare_first else 0)
    if rc != 0:
        raise RuntimeError("oracle run failed")
    return pos, vel, omg


def run_f64(p: Params, pos, vel, omg, steps: int):
    """The FP64 twin of run(): the same step in double from the given state
    (insertion order; omg.w holds no id here).  Returns (pos, vel, omg) as
    float64 n x 4 arrays in the input's row order (not cell-sorted) and the
    contact pairs of every state 0..steps-1 (the state each step integrates
    from)."""
    n = len(pos)
    P = np.array(pos, np.float64, copy=True)
    V = np.array(vel, np.float64, copy=True)
    W = np.array(omg, np.float64, copy=True)
    W[:, 3] = 0.0
    ids = np.arange(n, dtype=np.uint32)
    counts = np.zeros(max(steps, 1), np.uint64)
    rc = lib().sdo_run_f64(C.byref(p), n, _p(P), _p(V), _p(W), _p(ids), steps, _p(counts))
    if rc != 0:
        raise RuntimeError("oracle FP64 run failed")
    out = [np.empty_like(P), np.empty_like(V), np.empty_like(W)]
    for a, b in zip(out, (P, V, W)):
        a[ids] = b
    return out[0], out[1], out[2], counts[:steps].astype(np.int64)


def ensemble(pos, vel, omg):
    """Kinetic energy (translational + rotational, I = 0.4 m r^2), packing
    fraction (sphere volume over the volume of the spheres' bounding box)
    and contact count (pairs with |x_i - x_j| < r_i + r_j) of a sphere
    state, in double."""
    from scipy.spatial import cKDTree
    x = np.asarray(pos, np.float64)[:, :3]
    r = np.asarray(pos, np.float64)[:, 3]
    m = np.asarray(vel, np.float64)[:, 3]
    v = np.asarray(vel, np.float64)[:, :3]
    w = np.asarray(omg, np.float64)[:, :3]
    ke = float(0.5 * np.sum(m * np.sum(v * v, 1)) + 0.5 * np.sum(0.4 * m * r * r * np.sum(w * w, 1)))
    box = (x + r[:, None]).max(0) - (x - r[:, None]).min(0)
    phi = float(np.sum(4.0 / 3.0 * np.pi * r ** 3) / np.prod(box))
    pairs = np.array(sorted(cKDTree(x).query_pairs(2.0 * float(r.max()), output_type="ndarray").tolist()),
                     np.int64).reshape(-1, 2)
    if len(pairs):
        d = np.linalg.norm(x[pairs[:, 0]] - x[pairs[:, 1]], axis=1)
        pairs = pairs[d < r[pairs[:, 0]] + r[pairs[:, 1]]]
    return {"kinetic_energy": ke, "packing_fraction": phi, "contacts": int(len(pairs))}


def run_bodies(p: Params, pos, vel, omg, steps: int, bodies: dict, r0, body_of):
    """sdo_run_bodies: rigid clumps plus free spheres.  `bodies` holds float32
    arrays pos/vel/quat/omega/angmom (nb x 4), inv (nb x 3 x 4), first/count
    (uint32); they are copied and the stepped copies returned with the
    cell-sorted sphere state."""
    pos = np.array(pos, np.float32, copy=True)
    vel = np.array(vel, np.float32, copy=True)
    omg = np.array(omg, np.float32, copy=True)
    b = {k: np.array(bodies[k], np.float32, copy=True) for k in ("pos", "vel", "quat", "omega", "angmom", "inv")}
    first = np.ascontiguousarray(bodies["first"], np.uint32)
    count = np.ascontiguousarray(bodies["count"], np.uint32)
    r0 = np.ascontiguousarray(r0, np.float32)
    body_of = np.ascontiguousarray(body_of, np.int32)
    rc = lib().sdo_run_bodies(C.byref(p), len(pos), _p(pos), _p(vel), _p(omg), steps, len(first), _p(b["pos"]),
                              _p(b["vel"]), _p(b["quat"]), _p(b["omega"]), _p(b["angmom"]), _p(b["inv"]),
                              _p(first), _p(count), _p(r0), _p(body_of))
    if rc != 0:
        raise RuntimeError("oracle run failed")
    return pos, vel, omg, b


# ------------------------------------------------------------------ hulls
class HullParams(C.Structure):
    """sdo_hull_params (oracle/sd_oracle.h)."""
    _fields_ = [("lo", C.c_float * 3), ("hi", C.c_float * 3), ("kn", C.c_float), ("damp", C.c_float),
                ("mu", C.c_float), ("g", C.c_float * 3), ("dt", C.c_float), ("walls", C.c_int32)]


def hull_params(lo, hi, kn, damp, mu, g, dt, walls) -> HullParams:
    p = HullParams()
    for a in range(3):
        p.lo[a], p.hi[a], p.g[a] = lo[a], hi[a], g[a]
    p.kn, p.damp, p.mu, p.dt, p.walls = kn, damp, mu, dt, walls
    return p


def morton_ref(lo4, hi4, glo, ghi):
    lo4 = np.ascontiguousarray(lo4, np.float32)
    hi4 = np.ascontiguousarray(hi4, np.float32)
    out = np.empty(len(lo4), np.uint32)
    lib().sdo_morton_ref(len(lo4), _p(lo4), _p(hi4), _p(np.asarray(glo, np.float32)),
                         _p(np.asarray(ghi, np.float32)), _p(out))
    return out


def aabb_pairs(lo4, hi4):
    lo4 = np.ascontiguousarray(lo4, np.float32)
    hi4 = np.ascontiguousarray(hi4, np.float32)
    n = lib().sdo_aabb_pairs(len(lo4), _p(lo4), _p(hi4), None, 0)
    out = np.empty(max(n, 1), np.uint64)
    lib().sdo_aabb_pairs(len(lo4), _p(lo4), _p(hi4), _p(out), n)
    return out[:n].copy()


class Hulls:
    """Host copy of a hull scene (arrays as the oracle and the engine use them)."""

    def __init__(self, pos, vel, quat, omg, ang, iinv, vstart, vcount, verts):
        f = lambda a: np.ascontiguousarray(a, np.float32).copy()
        self.pos, self.vel, self.quat, self.omg, self.ang, self.iinv = map(f, (pos, vel, quat, omg, ang, iinv))
        self.vstart = np.ascontiguousarray(vstart, np.uint32)
        self.vcount = np.ascontiguousarray(vcount, np.uint32)
        self.verts = f(verts)

    @property
    def n(self):
        return len(self.pos)

    def copy(self):
        return Hulls(self.pos, self.vel, self.quat, self.omg, self.ang, self.iinv, self.vstart, self.vcount,
                     self.verts)

    def aabbs(self):
        lo = np.empty((self.n, 4), np.float32)
        hi = np.empty((self.n, 4), np.float32)
        ext = np.empty((self.n, 6), np.uint32)
        lib().sdo_hull_aabbs(self.n, _p(self.pos), _p(self.quat), _p(self.vstart), _p(self.vcount),
                             _p(self.verts), _p(lo), _p(hi), _p(ext))
        return lo, hi, ext

    def gjk_epa(self, a, b, seed=None):
        si = np.zeros(3, np.int32)
        res = np.zeros(10, np.float32)
        sd = None if seed is None else np.asarray(seed, np.float32)
        lib().sdo_gjk_epa(_p(self.pos), _p(self.quat), _p(self.iinv), _p(self.vstart), _p(self.vcount),
                          _p(self.verts), int(a), int(b), _p(sd), _p(si), _p(res))
        return {"status": int(si[0]), "iters": int(si[1]), "epa_iters": int(si[2]), "depth": float(res[0]),
                "normal": res[1:4].copy(), "point": res[4:7].copy(), "dir": res[7:10].copy()}

    def partners(self):
        lo, hi, _ = self.aabbs()
        off = np.empty(self.n + 1, np.uint32)
        cap = 2 * len(aabb_pairs(lo, hi)) + 1
        part = np.empty(cap, np.uint32)
        m = lib().sdo_hull_partners(self.n, _p(lo), _p(hi), _p(off), _p(part), cap)
        if m < 0:
            raise RuntimeError("partner capacity")
        return off, part[:m].copy()

    def step(self, p: HullParams, off=None, partners=None, seeds=None, record=False):
        """One step in place; returns per-entry (status, iters, dir) and per-body (force, torque)."""
        if off is None:
            off, partners = self.partners()
        m = len(partners)
        st = np.empty(max(m, 1), np.int32)
        it = np.empty(max(m, 1), np.int32)
        d4 = np.empty((max(m, 1), 4), np.float32)
        f = np.empty((self.n, 4), np.float32) if record else None
        t = np.empty((self.n, 4), np.float32) if record else None
        sd = None if seeds is None else np.ascontiguousarray(seeds, np.float32)
        lib().sdo_hull_step(C.byref(p), self.n, _p(self.pos), _p(self.vel), _p(self.quat), _p(self.omg),
                            _p(self.ang), _p(self.iinv), _p(self.vstart), _p(self.vcount), _p(self.verts),
                            _p(off), _p(partners), _p(sd), _p(st), _p(it), _p(d4), _p(f), _p(t))
        return {"off": off, "partners": partners, "status": st[:m], "iters": it[:m], "dir": d4[:m], "force": f,
                "torque": t}


def unsort(arr: np.ndarray, omg: np.ndarray) -> np.ndarray:
    """Back to insertion order by the ids in omg.w."""
    out = np.empty_like(arr)
    out[ids_of(omg)] = arr
    return out


def quat_from_matrix(R: np.ndarray) -> np.ndarray:
    """(s, x, y, z) of a proper rotation matrix (Shepperd's method), s >= 0."""
    t = np.trace(R)
    if t > 0:
        s = np.sqrt(t + 1.0) * 2
        q = [0.25 * s, (R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s]
    elif R[0, 0] > R[1, 1] and R[0, 0] > R[2, 2]:
        s = np.sqrt(1.0 + R[0, 0] - R[1, 1] - R[2, 2]) * 2
        q = [(R[2, 1] - R[1, 2]) / s, 0.25 * s, (R[0, 1] + R[1, 0]) / s, (R[0, 2] + R[2, 0]) / s]
    elif R[1, 1] > R[2, 2]:
        s = np.sqrt(1.0 + R[1, 1] - R[0, 0] - R[2, 2]) * 2
        q = [(R[0, 2] - R[2, 0]) / s, (R[0, 1] + R[1, 0]) / s, 0.25 * s, (R[1, 2] + R[2, 1]) / s]
    else:
        s = np.sqrt(1.0 + R[2, 2] - R[0, 0] - R[1, 1]) * 2
        q = [(R[1, 0] - R[0, 1]) / s, (R[0, 2] + R[2, 0]) / s, (R[1, 2] + R[2, 1]) / s, 0.25 * s]
    q = np.array(q)
    q /= np.linalg.norm(q)
    return q if q[0] >= 0 else -q


def matrix_from_quat(q) -> np.ndarray:
    s, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - s * z), 2 * (x * z + s * y)],
                     [2 * (x * y + s * z), 1 - 2 * (x * x + z * z), 2 * (y * z - s * x)],
                     [2 * (x * z - s * y), 2 * (y * z + s * x), 1 - 2 * (x * x + y * y)]])


def hulls_from_points(points, pos, quat, vel, mass, omega=None) -> Hulls:
    """Principal-frame hull bodies (numpy, FP64): centre of the points as
    equal point masses, their inertia diagonalised, vertices in the principal
    frame; the body's centre and orientation follow."""
    n = len(points)
    P = np.zeros((n, 4)); Q = np.zeros((n, 4)); V = np.zeros((n, 4)); W = np.zeros((n, 4))
    Lw = np.zeros((n, 4)); Ii = np.zeros((n, 4))
    vc, verts = [], []
    for i in range(n):
        p = np.asarray(points[i], np.float64)
        c = p.mean(axis=0)
        r = p - c
        m = float(mass[i])
        ms = m / len(p)
        I = ms * ((r * r).sum() * np.eye(3) - r.T @ r)
        lam, E = np.linalg.eigh(I)
        if np.linalg.det(E) < 0:
            E[:, 2] *= -1
        lam = np.maximum(lam, 1e-3 * lam.max())
        Ru = matrix_from_quat(quat[i])
        Rw = Ru @ E
        body = r @ E
        P[i, :3] = np.asarray(pos[i]) + Ru @ c
        P[i, 3] = m
        Q[i] = quat_from_matrix(Rw)
        V[i, :3] = vel[i]
        w = np.zeros(3) if omega is None else np.asarray(omega[i], np.float64)
        W[i, :3] = w
        Lw[i, :3] = Rw @ (lam * (Rw.T @ w))
        Ii[i, :3] = 1.0 / lam
        Ii[i, 3] = np.linalg.norm(body, axis=1).max()
        vc.append(len(p))
        verts.extend(body.tolist())
    vs = np.concatenate([[0], np.cumsum(vc)[:-1]]).astype(np.uint32)
    v4 = np.zeros((len(verts), 4))
    v4[:, :3] = verts
    return Hulls(P, V, Q, W, Lw, Ii, vs, np.array(vc, np.uint32), v4)


# ------------------------------------------------------ warm-start network
MLP_SIZES = {"W1": (64, 16), "b1": (64,), "W2": (64, 64), "b2": (64,), "W3": (16, 64), "b3": (16,)}
MLP_PARAMS = 6288


def mlp_unpack(p):
    out, o = {}, 0
    for k, shp in MLP_SIZES.items():
        n = int(np.prod(shp))
        out[k] = np.asarray(p[o:o + n], np.float64).reshape(shp)
        o += n
    return out


def mlp_pack(d):
    return np.concatenate([np.asarray(d[k], np.float32).ravel() for k in MLP_SIZES]).astype(np.float32)


def bf16(x):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def mlp_forward_bound(params, X, acc_eps=2.0 ** -23):
    """The forward pass of mlp_forward_backward with a per-element bound on
    how far a correct FP32-accumulating kernel can land from it: each
    pre-activation sums K exact BF16 x BF16 products and a bias in FP32, so
    it is off by at most (K + 1) * acc_eps * (sum of |terms|) (acc_eps =
    2^-23 admits truncating adds) plus what the previous layer's deviations
    carry through |W|; a BF16 rounding of relu(z) is monotone in z, so the
    activation can move at most to the roundings of the interval's ends.
    Returns (y (n, 3), bound (n, 3))."""
    P = mlp_unpack(params)
    W = [bf16(P["W1"]), bf16(P["W2"]), bf16(P["W3"])]
    b = [P["b1"], P["b2"], P["b3"]]
    H = bf16(X)
    dH = np.zeros_like(H)
    for layer in range(3):
        Wa = np.abs(W[layer])
        Z = H @ W[layer].T + b[layer]
        e = dH @ Wa.T + (W[layer].shape[1] + 1) * acc_eps * ((np.abs(H) + dH) @ Wa.T + np.abs(b[layer]))
        if layer == 2:
            break
        H = bf16(np.maximum(Z, 0))
        dH = np.maximum(np.abs(bf16(np.maximum(Z - e, 0)) - H), np.abs(bf16(np.maximum(Z + e, 0)) - H))
    skip = np.asarray(X, np.float64)[:, 8:11]
    Y = Z[:, :3] + skip
    # the residual add in FP32, rounded to nearest
    bound = e[:, :3] + 2.0 ** -24 * (np.abs(Z[:, :3]) + e[:, :3] + np.abs(skip))
    return Y, bound


def mlp_forward_backward(params, X, T, round_bf16=True, with_abs=False):
    """The network of sd_mlp.cu restated in float64: forward (rows of 16
    inputs; the output adds inputs 8..10, a residual over the previous
    direction) and the gradient of mean over rows of valid * (1 - y.t/|y|),
    with BF16 rounding where the tensor-core kernels round (inputs, hidden
    activations, output gradient and activation gradients).  Returns
    (y (n, 3), loss, grad (6288,)); with_abs adds the gradient's sums of
    |terms| per element (same packing), the scale of its rounding errors."""
    r = bf16 if round_bf16 else (lambda a: np.asarray(a, np.float64))
    P = mlp_unpack(params)
    W1, W2, W3 = r(P["W1"]), r(P["W2"]), r(P["W3"])
    n = len(X)
    Xb = r(X)
    Z1 = Xb @ W1.T + P["b1"]
    H1 = r(np.maximum(Z1, 0))
    Z2 = H1 @ W2.T + P["b2"]
    H2 = r(np.maximum(Z2, 0))
    Y = (H2 @ W3.T + P["b3"])[:, :3] + np.asarray(X, np.float64)[:, 8:11]  # residual over the previous direction
    t = np.asarray(T, np.float64)
    valid = t[:, 3] != 0
    nn = np.sqrt((Y * Y).sum(1) + 1e-8)
    c = (Y * t[:, :3]).sum(1) / nn
    loss = float((valid * (1 - c)).sum() / n)
    d = -(t[:, :3] - (c / nn)[:, None] * Y) / nn[:, None] / n
    d[~valid] = 0
    dY = np.zeros((n, 16))
    dY[:, :3] = r(d)
    dZ2 = r((dY @ W3) * (H2 > 0))
    dZ1 = r((dZ2 @ W2) * (H1 > 0))
    g = {"W3": dY.T @ H2, "b3": dY.sum(0), "W2": dZ2.T @ H1, "b2": dZ2.sum(0), "W1": dZ1.T @ Xb, "b1": dZ1.sum(0)}
    g["W3"][3:] = 0
    g["b3"][3:] = 0
    if not with_abs:
        return Y, loss, mlp_pack(g)
    a = np.abs
    ga = {"W3": a(dY).T @ a(H2), "b3": a(dY).sum(0), "W2": a(dZ2).T @ a(H1), "b2": a(dZ2).sum(0),
          "W1": a(dZ1).T @ a(Xb), "b1": a(dZ1).sum(0)}
    ga["W3"][3:] = 0
    ga["b3"][3:] = 0
    return Y, loss, mlp_pack(g), mlp_pack(ga)


def sap_sweep_ref(upperx, lowerx_sorted, uppery, lowery, idx_sorted):
    n = len(upperx)
    rows = np.empty((max(n, 1), 16), np.int32)
    f = lambda a: np.ascontiguousarray(a, np.float32)
    lib().sdo_sap_sweep_ref(n, _p(f(upperx)), _p(f(lowerx_sorted)), _p(f(uppery)), _p(f(lowery)),
                            _p(np.ascontiguousarray(idx_sorted, np.uint32)), _p(rows))
    return rows[:n]


def sap_process(pos4, radius=None):
    pos4 = np.ascontiguousarray(pos4, np.float32)
    n = len(pos4)
    rows = np.empty((max(n, 1), 16), np.int32)
    r = None if radius is None else np.ascontiguousarray(radius, np.float32)
    lib().sdo_sap_process(n, _p(pos4), _p(r), _p(rows))
    return rows[:n]


class Mesh(C.Structure):
    """sdo_mesh (oracle/sd_oracle.h)."""
    _fields_ = [("ntri", C.c_uint32), ("tri", C.c_void_p), ("patch", C.c_void_p), ("state", C.c_float * 24)]


def make_mesh(tris, patch, centre, state24):
    """Oracle mesh from world triangles at time 0 (mesh frame = world - centre)
    and the engine's pose state; keeps the arrays alive on the object."""
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3) - np.asarray(centre, np.float32)
    t4 = np.zeros((len(t), 3, 4), np.float32)
    t4[:, :, :3] = t
    t4 = np.ascontiguousarray(t4)
    pa = np.ascontiguousarray(np.arange(len(t)) if patch is None else patch, np.int32)
    m = Mesh()
    m.ntri = len(t)
    m.tri = t4.ctypes.data
    m.patch = pa.ctypes.data
    for k in range(24):
        m.state[k] = float(state24[k])
    m._keep = (t4, pa)
    return m


def make_mesh_frame(tri_frame, patch, state24):
    """Oracle mesh from triangles already in the mesh frame (as the engine
    stores them, sd_engine_get_mesh) and the engine's pose state."""
    t = np.asarray(tri_frame, np.float32).reshape(-1, 3, 3)
    t4 = np.zeros((len(t), 3, 4), np.float32)
    t4[:, :, :3] = t
    t4 = np.ascontiguousarray(t4)
    pa = np.ascontiguousarray(patch, np.int32)
    m = Mesh()
    m.ntri = len(t)
    m.tri = t4.ctypes.data
    m.patch = pa.ctypes.data
    for k in range(24):
        m.state[k] = float(state24[k])
    m._keep = (t4, pa)
    return m


def run_full(p: Params, pos, vel, omg, steps: int, bodies=None, r0=None, body_of=None, mesh=None):
    """sdo_run_full: optional clumps (as run_bodies) and an optional mesh."""
    pos = np.array(pos, np.float32, copy=True)
    vel = np.array(vel, np.float32, copy=True)
    omg = np.array(omg, np.float32, copy=True)
    if bodies is not None:
        b = {k: np.array(bodies[k], np.float32, copy=True) for k in ("pos", "vel", "quat", "omega", "angmom", "inv")}
        first = np.ascontiguousarray(bodies["first"], np.uint32)
        count = np.ascontiguousarray(bodies["count"], np.uint32)
        nb = len(first)
        args = [_p(b["pos"]), _p(b["vel"]), _p(b["quat"]), _p(b["omega"]), _p(b["angmom"]), _p(b["inv"]), _p(first),
                _p(count), _p(np.ascontiguousarray(r0, np.float32)), _p(np.ascontiguousarray(body_of, np.int32))]
    else:
        b, nb = None, 0
        args = [None] * 10
    rc = lib().sdo_run_full(C.byref(p), len(pos), _p(pos), _p(vel), _p(omg), steps, nb, *args,
                            None if mesh is None else C.byref(mesh))
    if rc != 0:
        raise RuntimeError("oracle run failed")
    return pos, vel, omg, b
