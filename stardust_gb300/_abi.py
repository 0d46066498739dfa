"""ctypes declarations of the C ABI in include/stardust.h.

The shared library is built in-tree (``stardust_gb300/libstardust_gb300.so``)
by ``stardust_gb300.build.build()``.  Loading fails loudly when it is
missing: there is no CPU fallback for any operation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libstardust_gb300.so"

# status codes (sd_status)
SD_OK = 0
SD_ERR_INVALID_ARG = 1
SD_ERR_CUDA = 2
SD_ERR_JSON = 3
SD_ERR_CAPACITY = 4
SD_ERR_ITER_LIMIT = 5
SD_ERR_STATE = 6
SD_ERR_IO = 7
SD_ERR_NOMEM = 8
SD_ERR_UNSUPPORTED = 9

STATUS_NAMES = {
    0: "SD_OK", 1: "SD_ERR_INVALID_ARG", 2: "SD_ERR_CUDA", 3: "SD_ERR_JSON",
    4: "SD_ERR_CAPACITY", 5: "SD_ERR_ITER_LIMIT", 6: "SD_ERR_STATE", 7: "SD_ERR_IO",
    8: "SD_ERR_NOMEM", 9: "SD_ERR_UNSUPPORTED",
}

SD_SNAPSHOT_CSV = 0
SD_SNAPSHOT_VTK = 1
SD_SNAPSHOT_CONTACTS = 0x1
SD_SNAPSHOT_MESH = 0x2
SD_ENGINE_SAP = 0
SD_ENGINE_SHP = 1
SD_DEVICE_CPU = 0
SD_DEVICE_GPU = 1

SD_FLAG_RECORD = 0x1

SD_FIELD_POSITION = 0
SD_FIELD_VELOCITY = 1
SD_FIELD_OMEGA = 2
SD_FIELD_FORCE = 3
SD_FIELD_TORQUE = 4
SD_FIELD_IDS = 5

SD_STAGE_CONTACT = 0
SD_STAGE_SORT = 1
SD_STAGE_REORDER = 2

SD_DEVERR_LOOKBACK_TIMEOUT = 0x1
SD_DEVERR_PAIR_OVERFLOW = 0x2
SD_DEVERR_BAD_INPUT = 0x4
SD_DEVERR_WAIT_TIMEOUT = 0x8

SD_BODY_POSITION = 0
SD_BODY_VELOCITY = 1
SD_BODY_QUATERNION = 2
SD_BODY_OMEGA = 3
SD_BODY_ANGMOM = 4
SD_BODY_INV_INERTIA = 5
SD_BODY_HULL_INV_INERTIA = 6
SD_BODY_FORCE = 7
SD_BODY_TORQUE = 8

SD_GJK_SEED_PLAIN = 0
SD_GJK_SEED_LEARNED = 1
SD_GJK_SEED_PREVIOUS = 2


class SdConfig(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("collision_engine", C.c_int32),
        ("device", C.c_int32),
        ("cuda_device", C.c_int32),
        ("domain", C.c_float),
        ("box_lo", C.c_float * 3),
        ("box_hi", C.c_float * 3),
        ("walls", C.c_int32),
        ("cell", C.c_float),
        ("kn", C.c_float),
        ("restitution", C.c_float),
        ("mu", C.c_float),
        ("gravity", C.c_float * 3),
        ("pair_capacity", C.c_uint64),
        ("flags", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class SdStats(C.Structure):
    _fields_ = [
        ("n_spheres", C.c_uint64),
        ("steps", C.c_uint64),
        ("contacts", C.c_uint64),
        ("kinetic_energy", C.c_double),
        ("momentum", C.c_double * 3),
        ("device_errors", C.c_uint32),
        ("n_cells", C.c_uint32),
        ("n_bodies", C.c_uint64),
        ("gjk_pairs", C.c_uint64),
        ("gjk_iters", C.c_uint64),
        ("epa_iters", C.c_uint64),
        ("moved_keys", C.c_uint64),
        ("step_kernels", C.c_uint64),
        ("list_builds", C.c_uint64),
        ("listed_steps", C.c_uint64),
    ]


class SdParams(C.Structure):
    _fields_ = [
        ("lo", C.c_float * 3), ("hi", C.c_float * 3), ("cell", C.c_float),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("kn", C.c_float), ("damp", C.c_float), ("mu", C.c_float),
        ("gravity", C.c_float * 3), ("dt", C.c_float), ("walls", C.c_int32),
        ("rmax", C.c_float), ("cell_z", C.c_float), ("z_div", C.c_int32),
    ]


P = C.c_void_p
U32 = C.c_uint32
U64 = C.c_uint64
I32 = C.c_int32
F32 = C.c_float
FP = C.POINTER(C.c_float)

# (name, restype-is-status, argtypes)
SIGNATURES = {
    "sd_config_default": [C.POINTER(SdConfig)],
    "sd_engine_create": [C.POINTER(SdConfig), C.POINTER(P)],
    "sd_engine_destroy": [P],
    "sd_last_error": [P, C.c_char_p, C.c_size_t],
    "sd_engine_add_spheres": [P, U64, P, P, P],
    "sd_engine_remove_spheres": [P, U64, P],
    "sd_engine_add_particle": [P, I32, F32, F32, F32, P, P],
    "sd_engine_add_clump": [P, U32, P, F32, P, P, P],
    "sd_engine_add_scene": [P, U64, P, P, P, P, P, F32],
    "sd_engine_add_mesh": [P, U32, P, P, P, P, F32],
    "sd_engine_get_mesh_state": [P, P],
    "sd_engine_get_mesh": [P, U64, P, P, P, C.POINTER(U64)],
    "sd_engine_write_snapshot": [P, C.c_char_p, I32, U32],
    "sd_stl_read": [C.c_char_p, U64, P, C.POINTER(U64)],
    "sd_mesh_patches": [U64, P, F32, P],
    "sd_engine_add_mesh_stl": [P, C.c_char_p, P, P, P, P, F32, F32],
    "sd_engine_get_bodies": [P, I32, P, C.c_size_t],
    "sd_engine_add_hull": [P, U32, P, F32, P, P, P, P],
    "sd_engine_get_hull_shapes": [P, P, P, P, U64, C.POINTER(U64)],
    "sd_engine_set_gjk_seed": [P, I32],
    "sd_engine_set_gjk_training": [P, I32, I32, F32],
    "sd_engine_hull_entries": [P, P, P, P, P, P, P, U64, C.POINTER(U64)],
    "sd_engine_mlp_params": [P, P, U64, I32],
    "sd_engine_mlp_forward": [P, P, P, U64],
    "sd_engine_mlp_train": [P, P, P, U64, I32, F32, P],
    "sd_sap_scratch_bytes": [U64, U64, C.POINTER(U64)],
    "sd_sap_pairs": [U64, P, P, P, U64, P, P, U64, P],
    "sd_sap_sweep": [U64, P, P, P, P, P, P, P],
    "sd_sap_process_collisions": [U64, P, P, P, P, U64, P],
    "sd_lbvh_scratch_bytes": [U64, U64, C.POINTER(U64)],
    "sd_lbvh_pairs": [U64, P, P, P, U64, P, P, U64, P],
    "sd_lbvh_morton": [U64, P, P, P, P, U64, P],
    "sd_engine_load_scene_json": [P, C.c_char_p],
    "sd_engine_prepare": [P],
    "sd_engine_step": [P, F32, I32],
    "sd_engine_update": [P, F32],
    "sd_engine_launch_stage": [P, I32, F32],
    "sd_tune_set": [C.c_char_p, I32],
    "sd_tune_get": [C.c_char_p, C.POINTER(I32)],
    "sd_engine_sync": [P],
    "sd_engine_get_state": [P, I32, P, C.c_size_t],
    "sd_engine_set_state": [P, I32, P, C.c_size_t],
    "sd_engine_device_ptr": [P, I32, C.POINTER(P)],
    "sd_engine_stream": [P, C.POINTER(P)],
    "sd_engine_get_pairs": [P, P, U64, C.POINTER(U64)],
    "sd_engine_stats": [P, C.POINTER(SdStats)],
    "sd_engine_params": [P, C.POINTER(SdParams)],
    "sd_engine_save_checkpoint": [P, C.c_char_p],
    "sd_engine_load_checkpoint": [P, C.c_char_p],
    "sd_hash_construct_collision_list": [U32, F32, P, P, P, P, P, P],
    "sd_sort_scratch_bytes": [U64, I32, C.POINTER(U64)],
    "sd_sort_pairs": [P, P, P, P, U64, I32, P, U64, P],
    "sd_hash_sort_collision_list": [P, P, P, P, U64, P, U64, P],
    "sd_sort_status": [P, P, C.POINTER(U32)],
    "sd_sort_pairs_noalloc": [P, P, P, P, U64, I32, P, P],
    "sd_hash_candidate_pairs": [P, P, P, U32, P, P, P, U64, P, P, U64, P],
    "sd_hash_pairs_scratch_bytes": [U64, C.POINTER(U64)],
    "sd_scene_lattice": [I32, I32, I32, F32, F32, P, F32, F32, F32, U64, P, P],
    "sd_scene_rsa": [U64, P, P, F32, F32, F32, F32, F32, F32, U64, U64, P, P, C.POINTER(C.c_double)],
}

_lib = None


class SdError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        self.status = status
        super().__init__(f"{where} -> {STATUS_NAMES.get(status, status)}: {message}")


def lib() -> C.CDLL:
    """The loaded C ABI library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
        l = C.CDLL(str(LIB_PATH))
        for name, args in SIGNATURES.items():
            fn = getattr(l, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _lib = l
    return _lib


def last_error(h=None) -> str:
    buf = C.create_string_buffer(1024)
    lib().sd_last_error(h, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int, where: str, h=None) -> None:
    if status != SD_OK:
        raise SdError(status, where, last_error(h))


def call(name: str, *args, h=None) -> None:
    check(getattr(lib(), name)(*args), name, h)


def tune_set(knob: str, value: int) -> None:
    """Set a process-wide launch knob (see sd_tune_set)."""
    call("sd_tune_set", knob.encode(), value)


def tune_get(knob: str) -> int:
    v = C.c_int32()
    call("sd_tune_get", knob.encode(), C.byref(v))
    return v.value
