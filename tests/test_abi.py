"""The C ABI library without a GPU: it loads, exports every declared entry
point, its structs match the ctypes mirror, and argument errors come back as
status codes (never exceptions or crashes)."""
from __future__ import annotations

import ctypes as C
import re
import subprocess

import numpy as np
import pytest

from conftest import REPO, cuda_available

HEADERS = sorted((REPO / "include").glob("*.h"))


def declared_functions():
    names = []
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"\b(bp_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "bp_solver_create" in names and "bp_solver_update" in names and "bp_grid_build" in names


def test_library_exports_every_declared_symbol(bp):
    lib = bp.abi.load()
    out = subprocess.run(["nm", "-D", "--defined-only", str(bp.abi.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\s[TW]\s+(\S+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for n in declared_functions():
        assert getattr(lib, n) is not None
    assert lib.bp_abi_version() == 1


def header_constants():
    """Every integer `#define BP_...` and enumerator `BP_... = value` of the
    headers."""
    out = {}
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for name, val in re.findall(r"#define\s+(BP_[A-Z0-9_]+)\s+(0x[0-9a-fA-F]+|[0-9]+)u?\b", text):
            out[name] = int(val, 0)
        for name, val in re.findall(r"\b(BP_[A-Z0-9_]+)\s*=\s*(0x[0-9a-fA-F]+|[0-9]+)\b", text):
            out[name] = int(val, 0)
    return out


def test_python_constants_match_header(bp):
    """The ctypes mirror's constants carry the header's values, and the
    header's walk and stage bits are all mirrored."""
    consts = header_constants()
    assert consts["BP_WALK_NO_PLANES"] == 0x40 and consts["BP_STAGE_ALL"] == 0x7FF
    mirrored = {k: getattr(bp.abi, k) for k in consts if hasattr(bp.abi, k)}
    wrong = {k: (v, consts[k]) for k, v in mirrored.items() if int(v) != consts[k]}
    assert not wrong, f"python value != header value: {wrong}"
    needed = [k for k in consts if k.startswith(("BP_WALK_", "BP_STAGE_", "BP_MODE_", "BP_FIELD_"))]
    missing = [k for k in needed if k not in mirrored]
    assert not missing, f"not mirrored in abi.py: {missing}"


def test_struct_layout_matches_header(bp, tmp_path):
    abi = bp.abi
    fields = {"bp_params": abi.BpParams, "bp_scene_desc": abi.BpSceneDesc, "bp_gradients": abi.BpGradients}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "brasspan.h"', "int main(void){"]
    for cname, py in fields.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{REPO / 'include'}", str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        struct, field, value = line.split()
        got[(struct, field)] = int(value)
    for cname, py in fields.items():
        assert got[(cname, "size")] == C.sizeof(py)
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_params_init_has_reference_literals(bp):
    p = bp.make_params()
    assert p.mode == bp.abi.BP_MODE_REFERENCE
    assert p.stage_mask == bp.abi.BP_STAGE_ALL
    assert p.gravity[1] == np.float32(-9.8)
    assert p.grid_dim == 512
    assert p.lambda_denominator == 15000.0 and p.scorr_n == 4
    assert p.delta_clamp == 5.0 and p.xsph_c == np.float32(0.0002)
    assert p.rotation_iterations == 20
    assert p.kernel_radius == np.float32(np.float32(2.3) * np.float32(0.05))


def _create(bp, scene, params):
    lib = bp.abi.load()
    desc, keep = bp.abi.scene_desc(scene)
    h = C.c_void_p()
    st = lib.bp_solver_create(C.byref(desc), C.byref(params) if params is not None else None, None, C.byref(h))
    return st, h


def test_create_rejects_bad_scenes(bp):
    abi = bp.abi
    s = bp.scenes.pbf_scene(3, 3, 3)
    p = bp.make_params(s)
    bad = bp.scenes.pbf_scene(3, 3, 3)
    bad.phases = bad.phases.copy()
    bad.phases[0] = 0
    assert _create(bp, bad, p)[0] == abi.BP_ERR_INVALID_ARGUMENT
    bad = bp.scenes.pbf_scene(3, 3, 3)
    bad.masses = bad.masses.copy()
    bad.masses[1] = -1.0
    assert _create(bp, bad, p)[0] == abi.BP_ERR_INVALID_ARGUMENT
    bad = bp.scenes.pbf_scene(3, 3, 3)
    bad.distance_pairs = np.array([[0, 10_000]], np.int32)
    bad.distance_params = np.array([[0.1, 1.0]], np.float32)
    assert _create(bp, bad, p)[0] == abi.BP_ERR_INVALID_ARGUMENT
    bad = bp.scenes.pbf_scene(3, 3, 3)
    bad.planes = np.zeros((17, 6), np.float32)
    assert _create(bp, bad, p)[0] == abi.BP_ERR_CAPACITY
    q = bp.make_params(s, grid_dim=48)
    assert _create(bp, s, q)[0] == abi.BP_ERR_INVALID_ARGUMENT
    q = bp.make_params(s, kernel_radius=1.0)
    assert _create(bp, s, q)[0] == abi.BP_ERR_INVALID_ARGUMENT
    assert _create(bp, s, None)[0] == abi.BP_ERR_INVALID_ARGUMENT
    assert b"params" in abi.load().bp_last_error_string()


def test_null_handles_are_errors(bp):
    lib = bp.abi.load()
    assert lib.bp_solver_step(None, C.c_float(0.01), 1, 1) == bp.abi.BP_ERR_INVALID_ARGUMENT
    assert lib.bp_solver_destroy(None) == bp.abi.BP_OK
    sz = C.c_size_t()
    assert lib.bp_grid_workspace_size(1000, 48, C.byref(sz)) == bp.abi.BP_ERR_INVALID_ARGUMENT
    assert lib.bp_grid_workspace_size(1000, 64, C.byref(sz)) == bp.abi.BP_OK and sz.value > 8000
    assert lib.bp_grid_build(None, -1, None, C.c_float(0.1), 64, None, None, None, None, None, None, 0) \
        == bp.abi.BP_ERR_INVALID_ARGUMENT


@pytest.mark.skipif(cuda_available(), reason="checks the no-device status path")
def test_create_without_device_reports_no_device(bp):
    s = bp.scenes.pbf_scene(3, 3, 3)
    st, _ = _create(bp, s, bp.make_params(s))
    assert st == bp.abi.BP_ERR_NO_DEVICE


def _create_batch(bp, scenes, params):
    lib = bp.abi.load()
    descs = (bp.abi.BpSceneDesc * len(scenes))()
    keep = []
    for k, s in enumerate(scenes):
        d, kk = bp.abi.scene_desc(s)
        descs[k] = d
        keep.append(kk)
    parr = (bp.abi.BpParams * len(params))(*params)
    h = C.c_void_p()
    st = lib.bp_batch_create(len(scenes), descs, parr, None, C.byref(h))
    if st == bp.abi.BP_OK:
        lib.bp_solver_destroy(h)
    return st, lib.bp_last_error_string().decode()


@pytest.mark.skipif(cuda_available(), reason="checks the argument validation that runs before the device check")
def test_batch_create_validates_scene_parameters(bp):
    a = bp.scenes.ensemble_member(200, seed=1)
    b = bp.scenes.ensemble_member(500, seed=2, rest_scale=0.9, gravity=12.0)
    pa, pb = bp.make_params(a), bp.make_params(b)
    assert pa.grid_dim != pb.grid_dim or pa.rest_density != pb.rest_density
    # rest density, gravity and grid dimension may differ: the call gets as far as the device
    assert _create_batch(bp, [a, b], [pa, pb])[0] == bp.abi.BP_ERR_NO_DEVICE
    # anything else may not
    pc = bp.make_params(b, xsph_c=0.01)
    st, msg = _create_batch(bp, [a, b], [pa, pc])
    assert st == bp.abi.BP_ERR_INVALID_ARGUMENT and "differ only" in msg
    pd = bp.make_params(b, neighbor_skin=0.1)
    assert _create_batch(bp, [a, b], [pa, pd])[0] == bp.abi.BP_ERR_INVALID_ARGUMENT
    assert _create_batch(bp, [], [])[0] == bp.abi.BP_ERR_INVALID_ARGUMENT


def test_batch_entry_points_reject_null_handles(bp):
    lib = bp.abi.load()
    first, count = C.c_int32(), C.c_int32()
    assert lib.bp_batch_scene_range(None, 0, C.byref(first), C.byref(count)) == bp.abi.BP_ERR_INVALID_ARGUMENT
    assert lib.bp_batch_step(None, C.c_float(0.01), 1, 1) == bp.abi.BP_ERR_INVALID_ARGUMENT


def test_ensemble_members_follow_the_configuration(bp):
    scenes = bp.scenes.dam_break_ensemble(seed=0, num_scenes=16)
    n = np.array([s.num_particles for s in scenes])
    assert n.min() >= 0.8 * 4096 and n.max() <= 1.1 * 262144
    rho = np.array([s.rest_density for s in scenes]) / 1000.0
    g = np.array([-s.gravity[1] for s in scenes])
    assert (rho >= 0.8 - 1e-6).all() and (rho <= 1.2 + 1e-6).all()
    assert (g >= 5.0).all() and (g <= 15.0).all()
    for s in scenes:  # the grid covers the box without aliasing
        assert s.grid_dim * s.cell_size >= s.planes[:, :3].max() - 1e-6
