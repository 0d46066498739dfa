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


def box_lattice(n_side: int = 16, seed: int = 0):
    """(pos4, vel4, EngineConfig, dt) of the jittered-lattice box."""
    edge = 0.64
    spacing = 2.2 * R_BOX
    extent = (n_side - 1) * spacing
    o = (edge - extent) / 2.0
    pos, vel = scene_lattice(n_side, n_side, n_side, spacing, 0.05 * R_BOX, (o, o, o), R_BOX, M_BOX, 0.1, seed)
    cfg = EngineConfig(box_lo=(0.0, 0.0, 0.0), box_hi=(edge, edge, edge), walls=0x3F, cell=2 * R_BOX,
                       kn=1e5, restitution=0.5, mu=0.3, gravity=(0.0, 0.0, -9.81))
    return pos, vel, cfg, 1e-5


def settling_rsa(n: int = 1 << 20, box=(1.0, 1.0, 2.0), seed: int = 0):
    """(pos4, vel4, EngineConfig, dt, volume_fraction) of the polydisperse settling box.

    Smaller n with a proportionally smaller box keeps the packing fraction.
    """
    rmed, sig, rmin, rmax = 0.005, 0.25, 0.0025, 0.01
    pos, vel, phi = scene_rsa(n, (0.0, 0.0, 0.0), box, rmed, sig, rmin, rmax, DENSITY, 0.0, seed)
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
