"""Python handle on the CPU oracle (TEST INFRASTRUCTURE ONLY).

* `OracleSolver`: the C restatement in oracle.c (liboracle.so), any mode.
* `RefSolver`: the reference's own kernels compiled for the host through
  oracle/refshim (oracle/_ref/libbrassref.so); reference parameters only.
* `RefCudaSolver`: the reference's own kernels compiled by nvcc for sm_103a
  and launched by the replay driver oracle/ref_cuda.cu
  (oracle/_ref/libbrassref_cuda.so); reference parameters only.

The two reference builds read the reference's kernel headers from
$BRASSPAN_REFERENCE/brasstower when that variable names a brass-pan checkout,
else from the staged copy oracle/_ref/src/brasstower (`make -C oracle stage`);
with neither, they are unavailable and the tests that need them skip.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this
module: as the oracle the GPU results are compared with, or as the timed CPU
baseline.
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
ORACLE_LIB = HERE / "_build" / "liboracle.so"
ORACLE64_LIB = HERE / "_build" / "liboracle64.so"
REF_LIB = HERE / "_ref" / "libbrassref.so"
REF_CUDA_LIB = HERE / "_ref" / "libbrassref_cuda.so"
STAGED_SRC = HERE / "_ref" / "src" / "brasstower"


def ref_source() -> Path | None:
    """Directory holding the reference's brasstower/ kernel headers, or None."""
    env = os.environ.get("BRASSPAN_REFERENCE")
    if env:
        p = Path(env) / "brasstower"
        if (p / "kernel" / "fluid.cuh").is_file():
            return p
    if (STAGED_SRC / "kernel" / "fluid.cuh").is_file():
        return STAGED_SRC
    return None


def stage_reference() -> bool:
    """Copies the reference headers the step needs into oracle/_ref/src
    (git-ignored) when $BRASSPAN_REFERENCE names a checkout; True if a
    staged copy exists afterwards."""
    env = os.environ.get("BRASSPAN_REFERENCE")
    if env and (Path(env) / "brasstower" / "kernel").is_dir():
        subprocess.run(["make", "-s", "-C", str(HERE), "stage", f"BRASSPAN_REFERENCE={env}"], check=True)
    return (STAGED_SRC / "kernel" / "fluid.cuh").is_file()


def _abi():
    mod = sys.modules.get("brasspan_gb300")
    if mod is not None:
        return mod.abi
    mod = sys.modules.get("_brasspan_abi")
    if mod is None:
        spec = importlib.util.spec_from_file_location("_brasspan_abi", REPO / "brass-pan_gb300" / "abi.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules["_brasspan_abi"] = mod
        spec.loader.exec_module(mod)
    return mod


def build_oracle(force: bool = False) -> Path:
    args = ["make", "-s", "-C", str(HERE), "all"]
    if force:
        args.insert(1, "-B")
    subprocess.run(args, check=True)
    return ORACLE_LIB


def build_ref(force: bool = False) -> Path | None:
    """Compiles the host build of the reference kernels; None without sources."""
    src = ref_source()
    if src is None:
        return None
    args = ["make", "-s", "-C", str(HERE), "ref", f"REF={src}"]
    if force:
        args.insert(1, "-B")
    subprocess.run(args, check=True)
    return REF_LIB


def build_ref_cuda(force: bool = False) -> Path | None:
    """Compiles the reference kernels for sm_103a with the replay driver
    (needs nvcc, no GPU); None without sources."""
    src = ref_source()
    if src is None:
        return None
    args = ["make", "-s", "-C", str(HERE), "ref_cuda", f"REF={src}"]
    if force:
        args.insert(1, "-B")
    subprocess.run(args, check=True)
    return REF_CUDA_LIB


_or = None
_or64 = None
_ref = None
_refcu = None


# The reference's literals (particlesolver.cuh, kernel/*.cuh, cubrasstower.cuh)
# as bp_params fields: the values bp_params_init writes, restated here so that
# the CPU reference arm can set up a run without loading the product library.
REFERENCE_LITERALS = dict(
    mode=0, stage_mask=0x7FF, solid_density_scale=2.0, lambda_denominator=15000.0, relaxation=300.0,
    scorr_k=0.0001, scorr_n=4, scorr_dq=0.03, delta_clamp=5.0, vorticity_eps=0.001, surface_tension=0.5,
    xsph_c=0.0002, friction_static=0.5, friction_dynamic=0.0, mass_scaling_k=2.0, wind_drag=10.0,
    wind_lift=100.0, rotation_iterations=20, neighbor_skin=0.0, walk_options=0x21, bending_stiffness=0.8)


def reference_params(scene, **overrides):
    """bp_params of `scene` with the reference's literals (what
    brasspan_gb300.make_params(scene) gives), then overrides; pure Python."""
    abi = _abi()
    p = abi.BpParams()
    for k, v in REFERENCE_LITERALS.items():
        setattr(p, k, v)
    p.particle_radius = scene.particle_radius
    p.kernel_radius = scene.kernel_radius
    p.cell_size = scene.cell_size
    p.grid_dim = scene.grid_dim
    p.rest_density = scene.rest_density
    for k in range(3):
        p.gravity[k] = scene.gravity[k]
    for k, v in overrides.items():
        if isinstance(getattr(p, k), C.Array):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, k, v)
    return p


def scenes_module():
    """brass-pan_gb300/scenes.py (pure Python scene builders) without
    importing the package or loading its library."""
    mod = sys.modules.get("brasspan_gb300")
    if mod is not None:
        return mod.scenes
    mod = sys.modules.get("_brasspan_scenes")
    if mod is None:
        spec = importlib.util.spec_from_file_location("_brasspan_scenes", REPO / "brass-pan_gb300" / "scenes.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules["_brasspan_scenes"] = mod
        spec.loader.exec_module(mod)
    return mod


def oracle_lib(precision: int = 32):
    """liboracle.so (fp32) or, precision=64, liboracle64.so (the FP64 host oracle)."""
    global _or, _or64
    cached = _or if precision == 32 else _or64
    if cached is None:
        path = ORACLE_LIB if precision == 32 else ORACLE64_LIB
        if not path.exists():
            build_oracle()
        lib = C.CDLL(str(path))
        if lib.or_real_size() != precision // 8:
            raise RuntimeError(f"{path.name}: expected {precision}-bit reals")
        abi = _abi()
        vp, i32, f32 = C.c_void_p, C.c_int32, C.c_float
        lib.or_create.restype = vp
        lib.or_create.argtypes = [C.POINTER(abi.BpSceneDesc), C.POINTER(abi.BpParams)]
        lib.or_destroy.argtypes = [vp]
        lib.or_set_params.argtypes = [vp, C.POINTER(abi.BpParams)]
        lib.or_update.argtypes = [vp, i32, f32, i32, i32, vp, vp]
        lib.or_get.argtypes = [vp, i32, vp]
        lib.or_set_state.argtypes = [vp, vp, vp]
        lib.or_set_full_state.argtypes = [vp, vp, vp, vp, vp]
        lib.or_set_threads.argtypes = [i32]
        lib.or_grid_build.argtypes = [i32, vp, f32, i32, vp, vp, vp, vp, vp]
        lib.or_neighbor_counts.argtypes = [i32, vp, f32, i32, f32, vp, vp, vp]
        lib.or_set_wind.argtypes = [vp, vp]
        lib.or_set_distance_params.argtypes = [vp, vp]
        if precision == 32:
            _or = lib
        else:
            _or64 = lib
        cached = lib
    return cached


def ref_lib():
    """The host build of the reference kernels, or None if it was not built."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            if build_ref() is None:
                return None
        lib = C.CDLL(str(REF_LIB))
        abi = _abi()
        vp, i32, f32 = C.c_void_p, C.c_int32, C.c_float
        lib.ref_create.restype = vp
        lib.ref_create.argtypes = [C.POINTER(abi.BpSceneDesc), f32, f32, f32, i32, f32]
        lib.ref_set_mass_scaling.argtypes = [vp, f32]
        lib.ref_destroy.argtypes = [vp]
        lib.ref_update.argtypes = [vp, i32, f32, i32, i32, i32, vp, vp]
        lib.ref_get.argtypes = [vp, i32, vp]
        lib.ref_set_threads.argtypes = [i32]
        lib.ref_grid_build.argtypes = [i32, vp, f32, i32, vp, vp, vp, vp, vp]
        lib.ref_neighbor_counts.argtypes = [i32, vp, f32, i32, f32, vp, vp, vp]
        _ref = lib
    return _ref


def ref_cuda_lib():
    """The reference kernels built for sm_103a with the replay driver, or None
    if they were not built (no reference sources) or no GPU is usable."""
    global _refcu
    if _refcu is None:
        if not REF_CUDA_LIB.exists():
            if build_ref_cuda() is None:
                return None
        lib = C.CDLL(str(REF_CUDA_LIB))
        abi = _abi()
        vp, i32, f32 = C.c_void_p, C.c_int32, C.c_float
        lib.refcu_create.restype = vp
        lib.refcu_create.argtypes = [C.POINTER(abi.BpSceneDesc), f32, f32, f32, i32, f32, f32]
        lib.refcu_destroy.argtypes = [vp]
        lib.refcu_update.argtypes = [vp, i32, f32, i32, i32, i32, vp, vp]
        lib.refcu_time_updates.argtypes = [vp, i32, i32, f32, i32, i32, vp, C.c_size_t, C.POINTER(f32)]
        lib.refcu_set_state.argtypes = [vp, vp, vp]
        lib.refcu_get.argtypes = [vp, i32, vp]
        lib.refcu_error.restype = i32
        _refcu = lib
    return _refcu


# field ids shared by or_get / ref_get / refcu_get
F_X, F_P, F_V, F_TO_ORIG, F_TO_NEW, F_LAMBDA, F_DENSITY, F_INVSCALED, F_SORTED_CELL, F_ROT, F_CM, \
    F_OMEGA, F_NORMAL, F_MASS, F_PHASE = range(15)


class _Base:
    n: int
    nb: int
    fdtype = np.float32  # element type of the float fields

    def _get(self, field):
        shapes = {F_X: (self.n, 3), F_P: (self.n, 3), F_V: (self.n, 3), F_OMEGA: (self.n, 3),
                  F_NORMAL: (self.n, 3), F_ROT: (self.nb, 4), F_CM: (self.nb, 3)}
        ints = {F_TO_ORIG, F_TO_NEW, F_SORTED_CELL, F_PHASE}
        shape = shapes.get(field, (self.n,))
        out = np.zeros(shape, np.int32 if field in ints else self.fdtype)
        if out.size:
            self._getter(self.h, field, out.ctypes.data)
        return out

    def get(self, field):
        return self._get(field)

    def positions(self, original_order=True):
        x = self._get(F_X)
        if not original_order:
            return x
        out = np.empty_like(x)
        out[self._get(F_TO_ORIG)] = x
        return out

    def velocities(self, original_order=True):
        v = self._get(F_V)
        if not original_order:
            return v
        out = np.empty_like(v)
        out[self._get(F_TO_ORIG)] = v
        return out

    def update(self, num_substeps, dt, iterations=2, picked=-1, picked_position=None, picked_velocity=None):
        pp = None if picked_position is None else np.ascontiguousarray(picked_position, np.float32)
        pv = None if picked_velocity is None else np.ascontiguousarray(picked_velocity, np.float32)
        self._update(num_substeps, dt, iterations, picked, pp, pv)


class OracleSolver(_Base):
    """oracle.c: the restatement, deterministic when single-threaded.
    precision=64 runs the FP64 host oracle (the same source in double): its
    fields come back as float64 and its state inputs are taken as float64."""

    def __init__(self, scene, params, threads: int = 1, precision: int = 32):
        self.lib = oracle_lib(precision)
        self.fdtype = np.float32 if precision == 32 else np.float64
        self.lib.or_set_threads(threads)
        abi = _abi()
        desc, keep = abi.scene_desc(scene)
        self.params = params
        self.h = self.lib.or_create(C.byref(desc), C.byref(params))
        self.n = scene.num_particles
        self.nb = int(len(scene.rigid_ranges))
        self._getter = self.lib.or_get

    def set_threads(self, threads):
        self.lib.or_set_threads(threads)

    def _update(self, nsub, dt, iters, picked, pp, pv):
        self.lib.or_update(self.h, nsub, C.c_float(dt), iters, picked,
                           None if pp is None else pp.ctypes.data, None if pv is None else pv.ctypes.data)

    def adopt(self, x_sorted, v_sorted, to_orig, rotations=None):
        """Takes over another solver's state, arrangement included."""
        x = np.ascontiguousarray(x_sorted, self.fdtype)
        v = np.ascontiguousarray(v_sorted, self.fdtype)
        t = np.ascontiguousarray(to_orig, np.int32)
        r = None if rotations is None else np.ascontiguousarray(rotations, self.fdtype)
        self.lib.or_set_full_state(self.h, x.ctypes.data, v.ctypes.data, t.ctypes.data,
                                   None if r is None else r.ctypes.data)

    def set_state(self, x_sorted=None, v_sorted=None):
        x = None if x_sorted is None else np.ascontiguousarray(x_sorted, self.fdtype)
        v = None if v_sorted is None else np.ascontiguousarray(v_sorted, self.fdtype)
        self.lib.or_set_state(self.h, None if x is None else x.ctypes.data, None if v is None else v.ctypes.data)

    def set_wind(self, wind):
        """The textbook wind vector, in this oracle's precision."""
        w = np.ascontiguousarray(wind, self.fdtype)
        self.lib.or_set_wind(self.h, w.ctypes.data)

    def set_distance_params(self, params):
        """(rest length, stiffness) of every distance constraint, [M][2]."""
        p = np.ascontiguousarray(params, self.fdtype)
        self.lib.or_set_distance_params(self.h, p.ctypes.data)

    def __del__(self):
        try:
            self.lib.or_destroy(self.h)
        except Exception:
            pass


class RefSolver(_Base):
    """The reference's own kernels on the host (reference parameters only)."""

    def __init__(self, scene, params, threads: int = 1):
        self.lib = ref_lib()
        if self.lib is None:
            raise RuntimeError("reference build unavailable (no reference checkout at build time)")
        self.lib.ref_set_threads(threads)
        abi = _abi()
        desc, keep = abi.scene_desc(scene)
        self.mask = params.stage_mask
        self.h = self.lib.ref_create(C.byref(desc), C.c_float(params.particle_radius),
                                     C.c_float(params.kernel_radius), C.c_float(params.cell_size),
                                     params.grid_dim, C.c_float(params.rest_density))
        self.lib.ref_set_mass_scaling(self.h, C.c_float(params.mass_scaling_k))
        self.n = scene.num_particles
        self.nb = int(len(scene.rigid_ranges))
        self._getter = self.lib.ref_get

    def _update(self, nsub, dt, iters, picked, pp, pv):
        self.lib.ref_update(self.h, nsub, C.c_float(dt), iters, self.mask, picked,
                            None if pp is None else pp.ctypes.data, None if pv is None else pv.ctypes.data)

    def __del__(self):
        try:
            self.lib.ref_destroy(self.h)
        except Exception:
            pass


class RefCudaSolver(_Base):
    """The reference's own kernels on the GPU (reference parameters only):
    nvcc-built for sm_103a, launched on the legacy default stream in the
    order of ParticleSolver::update, the stage mask and iteration count as
    parameters.  Float atomics make its sums order-dependent run to run."""

    def __init__(self, scene, params):
        self.lib = ref_cuda_lib()
        if self.lib is None:
            raise RuntimeError("reference CUDA build unavailable (no reference sources at build time)")
        abi = _abi()
        desc, keep = abi.scene_desc(scene)
        self.mask = params.stage_mask
        self.h = self.lib.refcu_create(C.byref(desc), C.c_float(params.particle_radius),
                                       C.c_float(params.kernel_radius), C.c_float(params.cell_size),
                                       params.grid_dim, C.c_float(params.rest_density),
                                       C.c_float(params.mass_scaling_k))
        if not self.h:
            raise RuntimeError(f"refcu_create failed (CUDA error {self.lib.refcu_error()})")
        self.n = scene.num_particles
        self.nb = int(len(scene.rigid_ranges))
        self._getter = self._get_checked

    def _get_checked(self, h, field, out):
        err = self.lib.refcu_get(h, field, out)
        if err:
            raise RuntimeError(f"reference CUDA step failed (CUDA error {err})")

    def _update(self, nsub, dt, iters, picked, pp, pv):
        err = self.lib.refcu_update(self.h, nsub, C.c_float(dt), iters, self.mask, picked,
                                    None if pp is None else pp.ctypes.data, None if pv is None else pv.ctypes.data)
        if err:
            raise RuntimeError(f"reference CUDA step failed (CUDA error {err})")

    def time_updates(self, frames, nsub, dt, iters, flush_ptr=None, flush_bytes=0):
        """Summed CUDA-event milliseconds of `frames` updates, L2 flushed by a
        write of flush_bytes to the device buffer flush_ptr before each."""
        ms = C.c_float(0.0)
        err = self.lib.refcu_time_updates(self.h, frames, nsub, C.c_float(dt), iters, self.mask, flush_ptr,
                                          flush_bytes, C.byref(ms))
        if err:
            raise RuntimeError(f"reference CUDA step failed (CUDA error {err})")
        return float(ms.value)

    def set_state(self, x_original, v_original):
        x = np.ascontiguousarray(x_original, np.float32)
        v = np.ascontiguousarray(v_original, np.float32)
        err = self.lib.refcu_set_state(self.h, x.ctypes.data, v.ctypes.data)
        if err:
            raise RuntimeError(f"refcu_set_state failed (CUDA error {err})")

    def close(self):
        if getattr(self, "h", None):
            self.lib.refcu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def grid_build(lib_kind: str, pos: np.ndarray, cell: float, D: int):
    """updateGridId + stable sort + findStartEndId on the host; returns
    (cell_ids, sorted_cell_ids, sorted_particle_ids, cell_start, cell_end)."""
    pos = np.ascontiguousarray(pos, np.float32)
    n = len(pos)
    lib = oracle_lib() if lib_kind == "oracle" else ref_lib()
    fn = lib.or_grid_build if lib_kind == "oracle" else lib.ref_grid_build
    cid = np.zeros(n, np.int32)
    scid = np.zeros(n, np.int32)
    spid = np.zeros(n, np.int32)
    cs = np.full(D ** 3, -1, np.int32)
    ce = np.full(D ** 3, -1, np.int32)
    fn(n, pos.ctypes.data, C.c_float(cell), D, cid.ctypes.data, scid.ctypes.data, spid.ctypes.data,
       cs.ctypes.data, ce.ctypes.data)
    return cid, scid, spid, cs, ce


def neighbor_counts(lib_kind: str, sorted_pos, cell, D, h, cs, ce):
    sorted_pos = np.ascontiguousarray(sorted_pos, np.float32)
    n = len(sorted_pos)
    lib = oracle_lib() if lib_kind == "oracle" else ref_lib()
    fn = lib.or_neighbor_counts if lib_kind == "oracle" else lib.ref_neighbor_counts
    out = np.zeros(n, np.int32)
    fn(n, sorted_pos.ctypes.data, C.c_float(cell), D, C.c_float(h), np.ascontiguousarray(cs).ctypes.data,
       np.ascontiguousarray(ce).ctypes.data, out.ctypes.data)
    return out
