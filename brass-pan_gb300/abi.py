"""ctypes view of the C ABI declared in include/brasspan.h.

The structures below mirror `bp_params` and `bp_scene_desc` field for field;
tests check their sizes and offsets against the C header.  `load()` opens the
in-tree `libbrasspan.so` and raises if it is missing: there is no fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libbrasspan.so"

# status codes
BP_OK = 0
BP_ERR_INVALID_ARGUMENT = 1
BP_ERR_CUDA = 2
BP_ERR_OUT_OF_MEMORY = 3
BP_ERR_CAPACITY = 4
BP_ERR_DEVICE_CHECK = 5
BP_ERR_NO_DEVICE = 6

BP_MODE_REFERENCE = 0
BP_MODE_TEXTBOOK = 1

BP_STAGE_PLANES = 0x001
BP_STAGE_WIND = 0x002
BP_STAGE_PARTICLE_COLLISION = 0x004
BP_STAGE_FLUID = 0x008
BP_STAGE_DISTANCE = 0x010
BP_STAGE_SHAPE_MATCHING = 0x020
BP_STAGE_IMMOVABLE = 0x040
BP_STAGE_VORTICITY = 0x080
BP_STAGE_AKINCI = 0x100
BP_STAGE_XSPH = 0x200
BP_STAGE_BENDING = 0x400
BP_STAGE_ALL = 0x7FF
BP_STAGE_REFERENCE_AS_SHIPPED = BP_STAGE_PLANES | BP_STAGE_VORTICITY | BP_STAGE_AKINCI | BP_STAGE_XSPH

BP_ORDER_SORTED = 0
BP_ORDER_ORIGINAL = 1

BP_DEVERR_NONFINITE = 0x1
BP_WALK_NO_STAGING = 0x1
BP_WALK_NO_SPLIT = 0x2
BP_WALK_NO_LISTS = 0x4
BP_WALK_NO_ALIAS_CLASSES = 0x8
BP_WALK_NO_FUSION = 0x10
BP_WALK_NO_CONTACT_CULLING = 0x20
BP_WALK_NO_PLANES = 0x40

(BP_FIELD_POSITIONS, BP_FIELD_NEW_POSITIONS, BP_FIELD_VELOCITIES, BP_FIELD_MAP_TO_ORIGINAL,
 BP_FIELD_MAP_TO_NEW, BP_FIELD_LAMBDAS, BP_FIELD_DENSITIES, BP_FIELD_SORTED_CELL_IDS,
 BP_FIELD_CELL_OFFSETS, BP_FIELD_RIGID_ROTATIONS, BP_FIELD_RIGID_CMS,
 BP_FIELD_INV_SCALED_MASSES) = range(12)
BP_FIELD_COUNT = 12


class BpParams(C.Structure):
    _fields_ = [
        ("mode", C.c_int32),
        ("stage_mask", C.c_int32),
        ("gravity", C.c_float * 3),
        ("particle_radius", C.c_float),
        ("kernel_radius", C.c_float),
        ("cell_size", C.c_float),
        ("grid_dim", C.c_int32),
        ("rest_density", C.c_float),
        ("solid_density_scale", C.c_float),
        ("lambda_denominator", C.c_float),
        ("relaxation", C.c_float),
        ("scorr_k", C.c_float),
        ("scorr_n", C.c_int32),
        ("scorr_dq", C.c_float),
        ("delta_clamp", C.c_float),
        ("vorticity_eps", C.c_float),
        ("surface_tension", C.c_float),
        ("xsph_c", C.c_float),
        ("friction_static", C.c_float),
        ("friction_dynamic", C.c_float),
        ("mass_scaling_k", C.c_float),
        ("wind_velocity", C.c_float * 3),
        ("wind_drag", C.c_float),
        ("wind_lift", C.c_float),
        ("rotation_iterations", C.c_int32),
        ("neighbor_skin", C.c_float),
        ("walk_options", C.c_int32),
        ("bending_stiffness", C.c_float),
        ("scan_block", C.c_int32),
        ("scan_persistent", C.c_int32),
        ("reserved", C.c_int32 * 3),
    ]


class BpSceneDesc(C.Structure):
    _fields_ = [
        ("num_particles", C.c_int32),
        ("positions", C.POINTER(C.c_float)),
        ("velocities", C.POINTER(C.c_float)),
        ("masses", C.POINTER(C.c_float)),
        ("phases", C.POINTER(C.c_int32)),
        ("group_ids", C.POINTER(C.c_int32)),
        ("num_planes", C.c_int32),
        ("planes", C.POINTER(C.c_float)),
        ("num_distance_constraints", C.c_int32),
        ("distance_pairs", C.POINTER(C.c_int32)),
        ("distance_params", C.POINTER(C.c_float)),
        ("num_wind_faces", C.c_int32),
        ("wind_faces", C.POINTER(C.c_int32)),
        ("num_rigid_bodies", C.c_int32),
        ("rigid_ranges", C.POINTER(C.c_int32)),
        ("rigid_rest_positions", C.POINTER(C.c_float)),
        ("num_immovables", C.c_int32),
        ("immovables", C.POINTER(C.c_int32)),
        ("num_bendings", C.c_int32),
        ("bendings", C.POINTER(C.c_int32)),
    ]


class BpStageTime(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_int32), ("total_ms", C.c_float)]


class BpGradients(C.Structure):
    _fields_ = [("positions", C.POINTER(C.c_float)), ("velocities", C.POINTER(C.c_float)),
                ("wind_velocity", C.POINTER(C.c_float)), ("distance_stiffness", C.POINTER(C.c_float)),
                ("distance_rest_length", C.POINTER(C.c_float))]


def _fptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _iptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int32))


def scene_desc(scene) -> tuple[BpSceneDesc, list]:
    """Builds a BpSceneDesc pointing into the numpy arrays of `scene`
    (an object with the attributes of scenes.Scene).  Returns the struct and
    the list of arrays that must stay alive while it is used."""
    keep = []

    def f32(a, shape_last=None):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float32)
        keep.append(a)
        return a

    def i32(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.int32)
        keep.append(a)
        return a

    d = BpSceneDesc()
    n = int(len(scene.positions))
    d.num_particles = n
    d.positions = _fptr(f32(scene.positions))
    d.velocities = _fptr(f32(scene.velocities)) if scene.velocities is not None else None
    d.masses = _fptr(f32(scene.masses))
    d.phases = _iptr(i32(scene.phases))
    d.group_ids = _iptr(i32(scene.group_ids)) if scene.group_ids is not None else None
    d.num_planes = int(len(scene.planes))
    d.planes = _fptr(f32(scene.planes)) if len(scene.planes) else None
    d.num_distance_constraints = int(len(scene.distance_pairs))
    d.distance_pairs = _iptr(i32(scene.distance_pairs)) if len(scene.distance_pairs) else None
    d.distance_params = _fptr(f32(scene.distance_params)) if len(scene.distance_pairs) else None
    d.num_wind_faces = int(len(scene.faces))
    d.wind_faces = _iptr(i32(scene.faces)) if len(scene.faces) else None
    d.num_rigid_bodies = int(len(scene.rigid_ranges))
    d.rigid_ranges = _iptr(i32(scene.rigid_ranges)) if len(scene.rigid_ranges) else None
    d.rigid_rest_positions = _fptr(f32(scene.rigid_rest)) if len(scene.rigid_ranges) else None
    d.num_immovables = int(len(scene.immovables))
    d.immovables = _iptr(i32(scene.immovables)) if len(scene.immovables) else None
    bendings = getattr(scene, "bendings", None)
    d.num_bendings = int(len(bendings)) if bendings is not None else 0
    d.bendings = _iptr(i32(bendings)) if d.num_bendings else None
    return d, keep


_lib = None

EXPORTS = [
    "bp_params_init", "bp_solver_create", "bp_solver_destroy", "bp_solver_update", "bp_solver_step",
    "bp_solver_set_params", "bp_solver_get_params", "bp_solver_query_original_particle_id",
    "bp_solver_query_new_particle_id",
    "bp_solver_get_particle_position", "bp_solver_copy_positions", "bp_solver_copy_velocities",
    "bp_solver_set_state", "bp_solver_snapshot_size", "bp_solver_snapshot_save", "bp_solver_snapshot_load",
    "bp_solver_field", "bp_solver_copy_field", "bp_solver_pack_particle_infos",
    "bp_solver_device_errors", "bp_solver_last_launch_count", "bp_solver_profile", "bp_solver_walk_stats", "bp_grid_workspace_size", "bp_grid_build",
    "bp_grid_reset", "bp_grid_build_static", "bp_batch_create", "bp_batch_step", "bp_batch_scene_range",
    "bp_solver_tape_begin", "bp_solver_backward", "bp_solver_tape_end", "bp_solver_autotune", "bp_grid_neighbor_counts", "bp_last_error_string", "bp_abi_version",
]


def load(path: Path | None = None):
    """Opens libbrasspan.so (built by build.py).  Raises if it is absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(p))
    vp, i32, f32, sz = C.c_void_p, C.c_int32, C.c_float, C.c_size_t
    pf, pi = C.POINTER(C.c_float), C.POINTER(C.c_int32)
    sig = {
        "bp_params_init": (None, [C.POINTER(BpParams), f32]),
        "bp_solver_create": (i32, [C.POINTER(BpSceneDesc), C.POINTER(BpParams), vp, C.POINTER(vp)]),
        "bp_solver_destroy": (i32, [vp]),
        "bp_solver_update": (i32, [vp, i32, f32, i32, i32, pf, pf]),
        "bp_solver_step": (i32, [vp, f32, i32, i32]),
        "bp_solver_set_params": (i32, [vp, C.POINTER(BpParams)]),
        "bp_solver_get_params": (i32, [vp, C.POINTER(BpParams)]),
        "bp_solver_query_original_particle_id": (i32, [vp, i32, pi]),
        "bp_solver_query_new_particle_id": (i32, [vp, i32, pi]),
        "bp_solver_get_particle_position": (i32, [vp, i32, pf]),
        "bp_solver_copy_positions": (i32, [vp, pf, i32]),
        "bp_solver_copy_velocities": (i32, [vp, pf, i32]),
        "bp_solver_set_state": (i32, [vp, pf, pf, i32]),
        "bp_solver_snapshot_size": (i32, [vp, C.POINTER(sz)]),
        "bp_solver_snapshot_save": (i32, [vp, vp, sz]),
        "bp_solver_snapshot_load": (i32, [vp, vp, sz]),
        "bp_solver_field": (i32, [vp, i32, C.POINTER(vp), C.POINTER(sz)]),
        "bp_solver_copy_field": (i32, [vp, i32, vp, sz]),
        "bp_solver_pack_particle_infos": (i32, [vp, vp]),
        "bp_solver_device_errors": (i32, [vp, C.POINTER(C.c_uint32)]),
        "bp_solver_last_launch_count": (i32, [vp, C.POINTER(C.c_int64)]),
        "bp_solver_profile": (i32, [vp, i32, f32, i32, i32, C.POINTER(BpStageTime), pi]),
        "bp_solver_walk_stats": (i32, [vp, i32, f32, i32, C.POINTER(C.c_uint64)]),
        "bp_grid_workspace_size": (i32, [i32, i32, C.POINTER(sz)]),
        "bp_grid_build": (i32, [vp, i32, vp, f32, i32, vp, vp, vp, vp, vp, vp, sz]),
        "bp_grid_reset": (i32, [vp, i32, vp, vp, vp]),
        "bp_grid_build_static": (i32, [vp, i32, vp, f32, i32, vp, vp, vp, vp, vp]),
        "bp_batch_create": (i32, [i32, vp, vp, vp, vp]),
        "bp_solver_tape_begin": (i32, [vp, i32]),
        "bp_solver_autotune": (i32, [vp, i32, f32, i32, vp, vp]),
        "bp_solver_backward": (i32, [vp, vp, vp, vp]),
        "bp_solver_tape_end": (i32, [vp]),
        "bp_batch_step": (i32, [vp, f32, i32, i32]),
        "bp_batch_scene_range": (i32, [vp, i32, vp, vp]),
        "bp_grid_neighbor_counts": (i32, [vp, i32, vp, f32, i32, f32, vp, vp, vp]),
        "bp_last_error_string": (C.c_char_p, []),
        "bp_abi_version": (i32, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class BrassPanError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"brasspan status {status}: {message}")
        self.status = status


def check(lib, status: int):
    if status != BP_OK:
        raise BrassPanError(status, lib.bp_last_error_string().decode())
    return status
