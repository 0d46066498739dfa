"""Seeded synthetic scenes of the DEM step's workloads.

``box_lattice`` is the 4,096-sphere plain-DEM box: 16^3 monodisperse spheres
(r = 0.01 m, m = 1e-3 kg) on a jittered cubic lattice (spacing 2.2 r, jitter
U[-0.05 r, 0.05 r]) centred in a 0.64 m walled cube, velocities U[-0.1, 0.1]
m/s, kn = 1e5 N/m, restitution 0.5, mu = 0.3, cell = 2 r, dt = 1e-5 s.

``settling_rsa`` is the 1,048,576-sphere polydisperse settling box: radii
lognormal (median 5 mm, sigma 0.25) clipped to [2.5, 10] mm, placed by random
sequential addition (largest first) in a walled 1 x 1 x 2 m box, at rest,
same material, density of the 4,096-sphere config (238.7 kg/m^3), cell = 2 x
max radius (50 x 50 x 100 cells), dt = 5e-6 s.  All 1,048,576 spheres of this
radius distribution fill 36.2 % of the box.

The reference ships no scene data beyond setup/star_test.json; these
generators stand in for its unseeded sandbox/testDEM.cpp:90-98 loop.
"""
from __future__ import annotations

import math

import numpy as np

from .engine import EngineConfig, scene_lattice, scene_rsa

R_BOX = 0.01
M_BOX = 1e-3
DENSITY = M_BOX / (4.0 / 3.0 * math.pi * R_BOX ** 3)


def box_lattice(n_side: int = 16, seed: int = 0, lattice=None):
    """(pos4, vel4, EngineConfig, dt) of the jittered-lattice box.  lattice:
    the builder (default the library's sd_scene_lattice; the oracle's copy
    gives the same spheres without loading the library)."""
    edge = 0.64
    spacing = 2.2 * R_BOX
    extent = (n_side - 1) * spacing
    o = (edge - extent) / 2.0
    pos, vel = (lattice or scene_lattice)(n_side, n_side, n_side, spacing, 0.05 * R_BOX, (o, o, o), R_BOX, M_BOX,
                                          0.1, seed)
    cfg = EngineConfig(box_lo=(0.0, 0.0, 0.0), box_hi=(edge, edge, edge), walls=0x3F, cell=2 * R_BOX,
                       kn=1e5, restitution=0.5, mu=0.3, gravity=(0.0, 0.0, -9.81))
    return pos, vel, cfg, 1e-5


def settling_rsa(n: int = 1 << 20, box=(1.0, 1.0, 2.0), seed: int = 0, rsa=None):
    """(pos4, vel4, EngineConfig, dt, volume_fraction) of the polydisperse settling box.

    Smaller n with a proportionally smaller box keeps the packing fraction.
    rsa: the packing builder (default the library's sd_scene_rsa; the
    oracle's copy gives the same spheres without loading the library).
    """
    rmed, sig, rmin, rmax = 0.005, 0.25, 0.0025, 0.01
    pos, vel, phi = (rsa or scene_rsa)(n, (0.0, 0.0, 0.0), box, rmed, sig, rmin, rmax, DENSITY, 0.0, seed)
    cfg = EngineConfig(box_lo=(0.0, 0.0, 0.0), box_hi=tuple(box), walls=0x3F, cell=2 * rmax, kn=1e5,
                       restitution=0.5, mu=0.3, gravity=(0.0, 0.0, -9.81))
    return pos, vel, cfg, 5e-6, phi


def scaled_box(n: int):
    """A 1 x 1 x 2 aspect box holding n spheres at the 1,048,576-sphere packing."""
    s = (n / float(1 << 20)) ** (1.0 / 3.0)
    return (1.0 * s, 1.0 * s, 2.0 * s)


def with_ids(omg: np.ndarray) -> np.ndarray:
    o = np.array(omg, np.float32, copy=True)
    o.view(np.uint32)[:, 3] = np.arange(len(o), dtype=np.uint32)
    return o


def _rotation(rng: np.random.Generator) -> np.ndarray:
    """A uniformly random rotation matrix (normalised Gaussian quaternion)."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    s, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - s * z), 2 * (x * z + s * y)],
                     [2 * (x * y + s * z), 1 - 2 * (x * x + z * z), 2 * (y * z - s * x)],
                     [2 * (x * z - s * y), 2 * (y * z + s * x), 1 - 2 * (x * x + y * y)]])


# body-frame sphere offsets of the clump shapes, in units of the sphere radius
CLUMP_SHAPES = {
    "dumbbell": np.array([[-0.8, 0, 0], [0.8, 0, 0]]),
    "triangle": np.array([[1.0, 0, 0], [-0.5, 0.866, 0], [-0.5, -0.866, 0]]),
    "tetra": np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]]) * 0.6,
    "cube": np.array([[i, j, k] for i in (-0.9, 0.9) for j in (-0.9, 0.9) for k in (-0.9, 0.9)]),
}


def clump_box(n_side: int = 8, free_fraction: float = 0.25, seed: int = 0, spacing: float = 5.0):
    """Rigid clumps and free spheres in a walled box.

    Slots of a jittered n_side^3 lattice (spacing x r; below about 5.2 the
    clumps of neighbouring slots can start in contact) each hold either a
    randomly oriented clump (dumbbell, triangle, tetrahedron or 2x2x2 cube of
    spheres of radius r = 0.01 m, overlapping, mass = density x summed sphere
    volumes) or, with probability free_fraction, one free sphere; velocities
    U[-0.2, 0.2] m/s, clump spins U[-20, 20] rad/s; box material as
    box_lattice.  Returns (clumps, free_pos4, free_vel4, EngineConfig, dt),
    clumps a list of (rel4, mass, com, vel, omega)."""
    rng = np.random.default_rng(seed)
    r = R_BOX
    spacing = spacing * r
    edge = n_side * spacing + 2 * r
    names = list(CLUMP_SHAPES)
    clumps, fp, fv = [], [], []
    vol = 4.0 / 3.0 * math.pi * r ** 3
    for i in range(n_side):
        for j in range(n_side):
            for k in range(n_side):
                c = np.array([i, j, k], float) * spacing + r + 0.5 * spacing
                c += rng.uniform(-0.1 * r, 0.1 * r, 3)
                v = rng.uniform(-0.2, 0.2, 3)
                if rng.random() < free_fraction:
                    fp.append([*c, r])
                    fv.append([*v, DENSITY * vol])
                    continue
                off = CLUMP_SHAPES[names[rng.integers(len(names))]] * r
                off = off @ _rotation(rng).T
                off -= off.mean(axis=0)
                rel = np.concatenate([off, np.full((len(off), 1), r)], axis=1).astype(np.float32)
                clumps.append((rel, float(DENSITY * vol * len(off)), tuple(c), tuple(v),
                               tuple(rng.uniform(-20.0, 20.0, 3))))
    cfg = EngineConfig(box_lo=(0.0, 0.0, 0.0), box_hi=(edge, edge, edge), walls=0x3F, cell=2 * r,
                       kn=1e5, restitution=0.5, mu=0.3, gravity=(0.0, 0.0, -9.81))
    return (clumps, np.array(fp, np.float32).reshape(-1, 4), np.array(fv, np.float32).reshape(-1, 4), cfg, 1e-5)


def add_clump_scene(eng, clumps, free_pos4, free_vel4) -> None:
    """Adds clump_box's bodies (ids first, in order) then its free spheres."""
    for rel, mass, com, vel, omega in clumps:
        eng.add_clump(rel, mass, com, vel, omega)
    if len(free_pos4):
        eng.add_spheres(free_pos4, free_vel4)


def _random_quats(rng: np.random.Generator, n: int) -> np.ndarray:
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 0] < 0] *= -1.0
    return q


def hull_box(n: int = 65_536, seed: int = 0, radius: float = 0.01, box=(1.0, 1.0, 1.0), vmax: float = 0.1,
             spacing: float | None = None):
    """Convex hulls dropped into a walled box.

    Each hull is the convex hull of 8-32 points sampled on the unit sphere
    with radial noise U[0.8, 1.2], scaled to `radius` (0.01 m: 0.02 m
    across), a random unit-quaternion orientation, mass = DENSITY x the
    volume of a sphere of the mean point radius.  Centres on a jittered
    lattice (spacing 2.5 x radius by default) filling the box from the
    floor up; velocities U[-vmax, vmax]; kn 1e5, restitution 0.5, mu 0.3,
    dt 1e-5.  Returns (points list, pos (n,3), quat (n,4), vel (n,3), mass
    (n,), EngineConfig, dt)."""
    rng = np.random.default_rng(seed)
    sp = spacing if spacing is not None else 2.5 * radius
    dims = [max(1, int((box[a] - 2 * radius) // sp)) for a in range(3)]
    if dims[0] * dims[1] * dims[2] < n:
        raise ValueError("box too small for n hulls at this spacing")
    pts, centres = [], []
    k = 0
    for iz in range(dims[2]):
        for iy in range(dims[1]):
            for ix in range(dims[0]):
                if k == n:
                    break
                centres.append([radius + (ix + 0.5) * sp, radius + (iy + 0.5) * sp, radius + (iz + 0.5) * sp])
                k += 1
    pos = np.array(centres) + rng.uniform(-0.05 * radius, 0.05 * radius, (n, 3))
    mass = np.empty(n)
    for i in range(n):
        m = int(rng.integers(8, 33))
        d = rng.normal(size=(m, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        p = d * rng.uniform(0.8, 1.2, (m, 1)) * radius
        pts.append(p.astype(np.float32))
        rm = float(np.linalg.norm(p, axis=1).mean())
        mass[i] = DENSITY * 4.0 / 3.0 * math.pi * rm ** 3
    quat = _random_quats(rng, n)
    vel = rng.uniform(-vmax, vmax, (n, 3))
    cfg = EngineConfig(box_lo=(0.0, 0.0, 0.0), box_hi=tuple(box), walls=0x3F, cell=4 * radius, kn=1e5,
                       restitution=0.5, mu=0.3, gravity=(0.0, 0.0, -9.81))
    return pts, pos.astype(np.float32), quat.astype(np.float32), vel.astype(np.float32), mass.astype(np.float32), \
        cfg, 1e-5


def batch_boxes(n_scenes: int = 512, seed: int = 0, n_min: int = 256, n_max: int = 65_536, median: int = 4096,
                sigma: float = 0.85, fraction: float = 0.35):
    """Independent sphere boxes for a batch: per scene a sphere count drawn
    lognormal (median 4,096, sigma 0.85, clipped to [256, 65,536]; ~3.1M
    spheres for 512 scenes), box_lattice's material and spheres (r = 0.01 m,
    m = 1e-3 kg) on a jittered cubic lattice whose spacing gives `fraction`
    of the box volume, its own seed, velocities U[-0.1, 0.1] m/s.  Returns
    (list of (pos4, vel4, lo, hi), EngineConfig, dt = 1e-5)."""
    rng = np.random.default_rng(seed)
    counts = np.clip(np.round(median * np.exp(sigma * rng.normal(size=n_scenes))), n_min, n_max).astype(int)
    r = R_BOX
    spacing = r * (4.0 / 3.0 * math.pi / fraction) ** (1.0 / 3.0)
    out = []
    for k, n in enumerate(counts):
        side = int(math.ceil(n ** (1.0 / 3.0)))
        pos, vel = scene_lattice(side, side, side, spacing, 0.05 * r, (0.5 * spacing,) * 3, r, M_BOX, 0.1,
                                 seed * 100_003 + k)
        edge = side * spacing
        out.append((pos[:n].copy(), vel[:n].copy(), (0.0, 0.0, 0.0), (edge, edge, edge)))
    cfg = EngineConfig(walls=0x3F, kn=1e5, restitution=0.5, mu=0.3, gravity=(0.0, 0.0, -9.81),
                       pair_capacity=1 << 22)
    return out, cfg, 1e-5


def drum_mesh(radius: float, length: float, n_around: int, n_along: int, n_rings: int, centre):
    """A closed cylinder along x: the side wall (n_around x n_along quads, two
    triangles each, patch 0) and two end caps (a fan plus n_rings - 1 rings of
    n_around sectors, patches 1 and 2).  Returns (tris (n, 3, 3), patch)."""
    cx, cy, cz = centre
    th = np.linspace(0.0, 2.0 * math.pi, n_around + 1)[:-1]
    xs = np.linspace(-0.5 * length, 0.5 * length, n_along + 1)
    ring = lambda x, r, k: (cx + x, cy + r * math.cos(th[k % n_around]), cz + r * math.sin(th[k % n_around]))
    tris, patch = [], []
    for i in range(n_along):
        for k in range(n_around):
            a, b = ring(xs[i], radius, k), ring(xs[i], radius, k + 1)
            c, d = ring(xs[i + 1], radius, k), ring(xs[i + 1], radius, k + 1)
            tris += [(a, b, d), (a, d, c)]
            patch += [0, 0]
    radii = np.linspace(0.0, radius, n_rings + 1)
    for side, x in ((1, -0.5 * length), (2, 0.5 * length)):
        centre_pt = (cx + x, cy, cz)
        for k in range(n_around):
            tris.append((centre_pt, ring(x, radii[1], k), ring(x, radii[1], k + 1)))
            patch.append(side)
        for j in range(1, n_rings):
            for k in range(n_around):
                a, b = ring(x, radii[j], k), ring(x, radii[j], k + 1)
                c, d = ring(x, radii[j + 1], k), ring(x, radii[j + 1], k + 1)
                tris += [(a, b, d), (a, d, c)]
                patch += [side, side]
    return np.array(tris, np.float32), np.array(patch, np.int32)


def drum_scene(n_spheres: int = 2_097_152, radius: float = 0.5, length: float = 0.5, n_around: int = 128,
               n_along: int = 65, n_rings: int = 8, r_range=(0.0012, 0.0024), clump_fraction: float = 0.1,
               omega: float = 2.0, density: float = 2500.0, seed: int = 0):
    """The rotating drum: a closed cylinder along x (20,480 triangles with the
    defaults) turning at omega rad/s, filled from the bottom with bodies on a
    jittered lattice (spacing 2.1 x the largest radius): single spheres with
    radii U[r_range], and clump_fraction of the bodies 4-sphere tetrahedral
    clumps (sphere radius U[r_min, 0.75 r_max], centres 0.6 r from the body
    centre, random orientation), until n_spheres spheres; density 2500
    kg/m^3, kn 1e5, restitution 0.5, mu 0.3, gravity -z, dt 2e-6 s.  Returns
    dict(tris, patch, centre, axis, omega, pos, vel, clumps, cfg, dt)."""
    rng = np.random.default_rng(seed)
    rmin, rmax = r_range
    centre = (0.5 * length, radius, radius)
    tris, patch = drum_mesh(radius, length, n_around, n_along, n_rings, centre)
    sp = 2.1 * rmax
    margin = 1.2 * rmax
    xs = np.arange(margin, length - margin + 1e-12, sp)
    ys = np.arange(margin, 2 * radius - margin + 1e-12, sp)
    zs = np.arange(margin, 2 * radius - margin + 1e-12, sp)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    sites = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    ok = (sites[:, 1] - centre[1]) ** 2 + (sites[:, 2] - centre[2]) ** 2 < (radius - margin) ** 2
    sites = sites[ok]
    sites = sites[np.argsort(sites[:, 2], kind="stable")]
    need = int(math.ceil(n_spheres / (1.0 + 3.0 * clump_fraction)))
    if need > len(sites):
        raise ValueError(f"the drum holds {len(sites)} bodies at this spacing, {need} requested")
    n_bodies = min(len(sites), int(need * 1.02) + 8)  # slack for the random clump share
    sites = sites[:n_bodies] + rng.uniform(-0.02 * rmax, 0.02 * rmax, (n_bodies, 3))
    is_clump = rng.random(n_bodies) < clump_fraction
    tet = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], float) / math.sqrt(3.0)
    pos, vel, clumps = [], [], []
    count = 0
    for b in range(n_bodies):
        if count >= n_spheres:
            break
        if is_clump[b] and count + 4 <= n_spheres:
            r = rng.uniform(rmin, 0.75 * rmax)
            off = (tet * 0.6 * r) @ _rotation(rng).T
            rel = np.concatenate([off, np.full((4, 1), r)], 1).astype(np.float32)
            mass = density * 4.0 / 3.0 * math.pi * r ** 3 * 4
            clumps.append((rel, float(mass), tuple(sites[b]), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)))
            count += 4
        else:
            r = rng.uniform(rmin, rmax)
            pos.append([*sites[b], r])
            vel.append([0.0, 0.0, 0.0, density * 4.0 / 3.0 * math.pi * r ** 3])
            count += 1
    cfg = EngineConfig(box_lo=(0.0, 0.0, 0.0), box_hi=(length, 2 * radius, 2 * radius), walls=0, cell=2 * rmax,
                       kn=1e5, restitution=0.5, mu=0.3, gravity=(0.0, 0.0, -9.81), pair_capacity=1 << 22)
    return {"tris": tris, "patch": patch, "centre": centre, "axis": (1.0, 0.0, 0.0), "omega": omega,
            "pos": np.array(pos, np.float32).reshape(-1, 4), "vel": np.array(vel, np.float32).reshape(-1, 4),
            "clumps": clumps, "cfg": cfg, "dt": 2e-6}


def add_drum_scene(eng, d, stl_path=None) -> None:
    """Adds drum_scene's clumps (ids first), spheres and mesh.  With
    stl_path the mesh goes through an STL file: written there (binary) and
    loaded with add_mesh_stl, whose smooth-face rule recovers the drum's
    three faces -- the same triangles and patches as the direct route."""
    for rel, mass, com, v, w in d["clumps"]:
        eng.add_clump(rel, mass, com, v, w)
    if len(d["pos"]):
        eng.add_spheres(d["pos"], d["vel"])
    if stl_path is None:
        eng.add_mesh(d["tris"], d["centre"], d["axis"], d["omega"], d["patch"])
    else:
        from .meshio import write_stl
        write_stl(stl_path, d["tris"])
        eng.add_mesh_stl(stl_path, centre=d["centre"], axis=d["axis"], omega=d["omega"], patch_angle=30.0)


def hopper_meshes(top: float = 0.12, outlet: float = 0.03, height: float = 0.08, z_outlet: float = 0.06,
                  tray: float = 0.16, tray_depth: float = 0.02):
    """A square hopper (four sloped walls, open top and outlet) above an
    open tray (floor and four low walls), centred on x = y = 0: (funnel
    (8, 3, 3), tray (10, 3, 3)) triangles, consistently wound."""
    a, b = 0.5 * top, 0.5 * outlet
    zt, zb = z_outlet + height, z_outlet
    ring_t = [(-a, -a, zt), (a, -a, zt), (a, a, zt), (-a, a, zt)]
    ring_b = [(-b, -b, zb), (b, -b, zb), (b, b, zb), (-b, b, zb)]
    funnel = []
    for k in range(4):
        p0, p1, q0, q1 = ring_b[k], ring_b[(k + 1) % 4], ring_t[k], ring_t[(k + 1) % 4]
        funnel += [(p0, p1, q1), (p0, q1, q0)]
    c = 0.5 * tray
    floor = [(-c, -c, 0.0), (c, -c, 0.0), (c, c, 0.0), (-c, c, 0.0)]
    rim = [(x, y, tray_depth) for x, y, _ in floor]
    tray_t = [(floor[0], floor[2], floor[1]), (floor[0], floor[3], floor[2])]
    for k in range(4):
        p0, p1, q0, q1 = floor[k], floor[(k + 1) % 4], rim[k], rim[(k + 1) % 4]
        tray_t += [(p0, p1, q1), (p0, q1, q0)]
    return np.array(funnel, np.float32), np.array(tray_t, np.float32)
