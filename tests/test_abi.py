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


def test_struct_layout_matches_header(bp, tmp_path):
    abi = bp.abi
    fields = {"bp_params": abi.BpParams, "bp_scene_desc": abi.BpSceneDesc}
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
