"""stardust-gb300: a GB300-native (sm_103a) DEM step behind a C ABI.

The product is ``libstardust_gb300.so`` (C ABI: include/stardust.h).  This
package builds it (``stardust_gb300.build``) and mirrors the reference's
engine and operator classes over it (``stardust_gb300.engine``).
"""
from . import _abi
from ._abi import SdError, lib
from .engine import (BoundingVolumes, DEMEngine, EngineConfig, SpatialPartition, SweepAndPrune, add_hull_scene,
                     scene_lattice, scene_rsa)
from .meshio import mesh_patches, read_stl, write_stl

__all__ = ["BoundingVolumes", "DEMEngine", "EngineConfig", "SpatialPartition", "SweepAndPrune", "SdError",
           "add_hull_scene", "lib", "mesh_patches", "read_stl", "write_stl",
           "scene_lattice", "scene_rsa", "_abi"]
