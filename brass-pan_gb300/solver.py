"""Python mirror of the reference's ParticleSolver interface over the C ABI.

Method names follow brasstower/particlesolver.cuh (update, queryOriginalParticleId,
queryNewParticleId, getParticlePosition) so host code written against the
reference ports line for line.  Every call goes through libbrasspan.so; there
is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .scenes import Scene


def make_params(scene: Scene | None = None, mode: int = abi.BP_MODE_REFERENCE, stage_mask: int | None = None,
                **overrides) -> abi.BpParams:
    """bp_params with the reference's literals, the scene's geometry, then overrides."""
    lib = abi.load()
    p = abi.BpParams()
    radius = scene.particle_radius if scene is not None else 0.05
    lib.bp_params_init(C.byref(p), C.c_float(radius))
    if scene is not None:
        p.kernel_radius = scene.kernel_radius
        p.cell_size = scene.cell_size
        p.grid_dim = scene.grid_dim
        p.rest_density = scene.rest_density
        for k in range(3):
            p.gravity[k] = scene.gravity[k]
    p.mode = mode
    if stage_mask is not None:
        p.stage_mask = stage_mask
    for k, v in overrides.items():
        if isinstance(getattr(p, k), C.Array):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, k, v)
    return p


class ParticleSolver:
    """One solver handle on the current CUDA device."""

    def __init__(self, scene: Scene, params: abi.BpParams | None = None, stream: int | None = None):
        self.lib = abi.load()
        self.scene = scene
        self.params = params if params is not None else make_params(scene)
        desc, self._keep = abi.scene_desc(scene)
        h = C.c_void_p()
        abi.check(self.lib, self.lib.bp_solver_create(C.byref(desc), C.byref(self.params),
                                                      C.c_void_p(stream) if stream else None, C.byref(h)))
        self.handle = h
        self.n = scene.num_particles

    # -- reference interface ------------------------------------------------------
    def update(self, num_substeps: int, dt: float, iterations: int = 2, picked_original_id: int = -1,
               picked_position=(0.0, 0.0, 0.0), picked_velocity=(0.0, 0.0, 0.0)):
        pp = (C.c_float * 3)(*picked_position)
        pv = (C.c_float * 3)(*picked_velocity)
        abi.check(self.lib, self.lib.bp_solver_update(self.handle, num_substeps, C.c_float(dt), iterations,
                                                      picked_original_id, pp, pv))

    def step(self, dt: float, substeps: int, iterations: int):
        abi.check(self.lib, self.lib.bp_solver_step(self.handle, C.c_float(dt), substeps, iterations))

    def queryOriginalParticleId(self, sorted_index: int) -> int:
        out = C.c_int32()
        abi.check(self.lib, self.lib.bp_solver_query_original_particle_id(self.handle, sorted_index, C.byref(out)))
        return out.value

    def queryNewParticleId(self, original_id: int) -> int:
        out = C.c_int32()
        abi.check(self.lib, self.lib.bp_solver_query_new_particle_id(self.handle, original_id, C.byref(out)))
        return out.value

    def getParticlePosition(self, sorted_index: int) -> np.ndarray:
        out = (C.c_float * 3)()
        abi.check(self.lib, self.lib.bp_solver_get_particle_position(self.handle, sorted_index, out))
        return np.array(out[:], np.float32)

    # -- state access ----------------------------------------------------------------
    def positions(self, order: int = abi.BP_ORDER_ORIGINAL) -> np.ndarray:
        out = np.empty((self.n, 3), np.float32)
        abi.check(self.lib, self.lib.bp_solver_copy_positions(
            self.handle, out.ctypes.data_as(C.POINTER(C.c_float)), order))
        return out

    def velocities(self, order: int = abi.BP_ORDER_ORIGINAL) -> np.ndarray:
        out = np.empty((self.n, 3), np.float32)
        abi.check(self.lib, self.lib.bp_solver_copy_velocities(
            self.handle, out.ctypes.data_as(C.POINTER(C.c_float)), order))
        return out

    def set_state(self, positions=None, velocities=None, order: int = abi.BP_ORDER_ORIGINAL):
        x = None if positions is None else np.ascontiguousarray(positions, np.float32)
        v = None if velocities is None else np.ascontiguousarray(velocities, np.float32)
        abi.check(self.lib, self.lib.bp_solver_set_state(
            self.handle, None if x is None else x.ctypes.data_as(C.POINTER(C.c_float)),
            None if v is None else v.ctypes.data_as(C.POINTER(C.c_float)), order))

    def set_params(self, params: abi.BpParams):
        """bp_solver_set_params: new parameters from the next update on."""
        abi.check(self.lib, self.lib.bp_solver_set_params(self.handle, C.byref(params)))
        self.params = params

    def snapshot(self) -> bytes:
        """Checkpoint: the whole state as bytes (bp_solver_snapshot_save)."""
        size = C.c_size_t()
        abi.check(self.lib, self.lib.bp_solver_snapshot_size(self.handle, C.byref(size)))
        buf = C.create_string_buffer(size.value)
        abi.check(self.lib, self.lib.bp_solver_snapshot_save(self.handle, buf, size.value))
        return buf.raw

    def restore(self, snap: bytes):
        """Resume from snapshot() bytes of a solver of the same scene."""
        buf = C.create_string_buffer(bytes(snap), len(snap))
        abi.check(self.lib, self.lib.bp_solver_snapshot_load(self.handle, buf, len(snap)))

    _DTYPES = {
        abi.BP_FIELD_POSITIONS: (np.float32, 4), abi.BP_FIELD_NEW_POSITIONS: (np.float32, 4),
        abi.BP_FIELD_VELOCITIES: (np.float32, 4), abi.BP_FIELD_MAP_TO_ORIGINAL: (np.int32, 1),
        abi.BP_FIELD_MAP_TO_NEW: (np.int32, 1), abi.BP_FIELD_LAMBDAS: (np.float32, 1),
        abi.BP_FIELD_DENSITIES: (np.float32, 1), abi.BP_FIELD_SORTED_CELL_IDS: (np.int32, 1),
        abi.BP_FIELD_CELL_OFFSETS: (np.int32, 1), abi.BP_FIELD_RIGID_ROTATIONS: (np.float32, 4),
        abi.BP_FIELD_RIGID_CMS: (np.float32, 4), abi.BP_FIELD_INV_SCALED_MASSES: (np.float32, 1),
    }

    def field_ptr(self, field: int) -> tuple[int, int]:
        ptr = C.c_void_p()
        nbytes = C.c_size_t()
        abi.check(self.lib, self.lib.bp_solver_field(self.handle, field, C.byref(ptr), C.byref(nbytes)))
        return ptr.value or 0, nbytes.value

    def field(self, field: int) -> np.ndarray:
        dt, width = self._DTYPES[field]
        _, nbytes = self.field_ptr(field)
        out = np.empty(nbytes // 4, dt)
        if nbytes:
            abi.check(self.lib, self.lib.bp_solver_copy_field(self.handle, field, out.ctypes.data, nbytes))
        return out.reshape(-1, width) if width > 1 else out

    def device_errors(self) -> int:
        out = C.c_uint32()
        abi.check(self.lib, self.lib.bp_solver_device_errors(self.handle, C.byref(out)))
        return out.value

    def last_launch_count(self) -> int:
        out = C.c_int64()
        abi.check(self.lib, self.lib.bp_solver_last_launch_count(self.handle, C.byref(out)))
        return out.value

    def profile(self, num_substeps: int, dt: float, iterations: int) -> dict[str, tuple[int, float]]:
        """One real update with a CUDA event after every kernel: {kernel: (launches, total ms)}."""
        cap = 64
        buf = (abi.BpStageTime * cap)()
        count = C.c_int32()
        abi.check(self.lib, self.lib.bp_solver_profile(self.handle, num_substeps, C.c_float(dt), iterations, cap,
                                                       buf, C.byref(count)))
        return {buf[k].name.decode(): (buf[k].launches, buf[k].total_ms) for k in range(min(cap, count.value))}

    def walk_stats(self, num_substeps: int, dt: float, iterations: int) -> dict[str, int]:
        """One real update counting the neighbour walks of all scan passes by kind."""
        out = (C.c_uint64 * 5)()
        abi.check(self.lib, self.lib.bp_solver_walk_stats(self.handle, num_substeps, C.c_float(dt), iterations, out))
        return {"listed": int(out[0]), "cells_no_list": int(out[1]), "cells_moved_cell": int(out[2]),
                "cells_displaced": int(out[3]), "alias_classes": int(out[4])}

    def autotune(self, num_substeps: int, dt: float, iterations: int) -> tuple[int, list[float]]:
        """Keep the fastest walk variant and scan launch shape for this scene;
        returns the walk options and the trial times (ms) of the thirteen
        candidates (bp_solver_autotune); the launch shape chosen is in
        self.params (scan_block, scan_persistent)."""
        opt = C.c_int32()
        ms = (C.c_float * 13)()
        abi.check(self.lib, self.lib.bp_solver_autotune(self.handle, num_substeps, C.c_float(dt), iterations,
                                                        C.byref(opt), ms))
        abi.check(self.lib, self.lib.bp_solver_get_params(self.handle, C.byref(self.params)))
        return opt.value, list(ms)

    # -- differentiable rollouts ------------------------------------------------------
    def tape_begin(self, checkpoint_every: int = 10):
        """Record the following updates for backward()."""
        abi.check(self.lib, self.lib.bp_solver_tape_begin(self.handle, checkpoint_every))

    def tape_end(self):
        abi.check(self.lib, self.lib.bp_solver_tape_end(self.handle))

    def backward(self, grad_positions=None, grad_velocities=None) -> dict[str, np.ndarray]:
        """Gradients of a loss of the final state (dL/dx, dL/dv: [N][3], original
        order) with respect to the state at tape_begin and the parameters."""
        fp = C.POINTER(C.c_float)

        def arr(a):
            return None if a is None else np.ascontiguousarray(a, np.float32).reshape(self.n, 3)

        gx, gv = arr(grad_positions), arr(grad_velocities)
        m = int(self.scene.num_distance_constraints) if self.scene is not None else 0
        out = {"positions": np.zeros((self.n, 3), np.float32), "velocities": np.zeros((self.n, 3), np.float32),
               "wind_velocity": np.zeros(3, np.float32), "distance_stiffness": np.zeros(m, np.float32),
               "distance_rest_length": np.zeros(m, np.float32)}
        g = abi.BpGradients()
        for k, v in out.items():
            setattr(g, k, v.ctypes.data_as(fp) if v.size else None)
        abi.check(self.lib, self.lib.bp_solver_backward(
            self.handle, None if gx is None else gx.ctypes.data_as(fp),
            None if gv is None else gv.ctypes.data_as(fp), C.byref(g)))
        return out

    def pack_particle_infos(self, device_ptr: int):
        abi.check(self.lib, self.lib.bp_solver_pack_particle_infos(self.handle, C.c_void_p(device_ptr)))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.bp_solver_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class BatchSolver(ParticleSolver):
    """Many independent scenes stepped together (bp_batch_create).

    The handle is a solver over the scenes' particles in scene order; every
    ParticleSolver method applies to all of them at once, and scene_positions /
    scene_velocities slice one scene out."""

    def __init__(self, scenes: list[Scene], params: list[abi.BpParams] | None = None, stream: int | None = None):
        self.lib = abi.load()
        self.scenes = list(scenes)
        self.scene = None
        plist = params if params is not None else [make_params(s) for s in self.scenes]
        self.params_list = list(plist)
        self.params = self.params_list[0]
        descs = (abi.BpSceneDesc * len(self.scenes))()
        self._keep = []
        for k, s in enumerate(self.scenes):
            d, keep = abi.scene_desc(s)
            descs[k] = d
            self._keep.append(keep)
        parr = (abi.BpParams * len(self.params_list))(*self.params_list)
        h = C.c_void_p()
        abi.check(self.lib, self.lib.bp_batch_create(len(self.scenes), descs, parr,
                                                     C.c_void_p(stream) if stream else None, C.byref(h)))
        self.handle = h
        self.n = sum(s.num_particles for s in self.scenes)
        self.ranges = []
        for k in range(len(self.scenes)):
            first, count = C.c_int32(), C.c_int32()
            abi.check(self.lib, self.lib.bp_batch_scene_range(self.handle, k, C.byref(first), C.byref(count)))
            self.ranges.append((first.value, count.value))

    def step(self, dt: float, substeps: int, iterations: int):
        abi.check(self.lib, self.lib.bp_batch_step(self.handle, C.c_float(dt), substeps, iterations))

    def scene_positions(self, k: int) -> np.ndarray:
        first, count = self.ranges[k]
        return self.positions()[first:first + count]

    def scene_velocities(self, k: int) -> np.ndarray:
        first, count = self.ranges[k]
        return self.velocities()[first:first + count]
