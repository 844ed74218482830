"""The reference's own CUDA step (its kernel headers built for sm_103a and
replayed by oracle/ref_cuda.cu) against the GB300 solver and the oracle.

This pins the comparator the benchmark times: from the same initial state,
one substep of the reference's CUDA build agrees with the GB300 solver and
with the oracle to max |dx| <= 1e-4 * h, and its neighbour search (sorted cell
ids, sorted order) is identical.  The reference sums with float atomics in an
order that changes from run to run, so rounding differs; nothing else may."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import fluid_scene, small_mixed_scene

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


@pytest.fixture(scope="module")
def refcuda(oracle, gpu):
    if oracle.ref_cuda_lib() is None:
        pytest.skip("the reference's sources were not available to build its CUDA step")
    return oracle


def _one_substep(bp, oracle, scene, params, iterations=4, substeps=1):
    g = bp.ParticleSolver(scene, params)
    r = oracle.RefCudaSolver(scene, params)
    o = oracle.OracleSolver(scene, params)
    sdt = DT / 2
    try:
        for s in (g, r, o):
            s.update(substeps, sdt * substeps, iterations)
        out = {
            "gpu": g.positions(), "ref": r.positions(), "oracle": o.positions(),
            "gpu_v": g.velocities(), "ref_v": r.velocities(),
            "keys_equal": np.array_equal(g.field(bp.abi.BP_FIELD_SORTED_CELL_IDS), r.get(oracle.F_SORTED_CELL)),
            "order_equal": np.array_equal(g.field(bp.abi.BP_FIELD_MAP_TO_ORIGINAL), r.get(oracle.F_TO_ORIG)),
        }
    finally:
        g.close()
        r.close()
    return out, sdt


@pytest.mark.parametrize("name", ["fluid", "mixed"])
def test_reference_cuda_substep_matches_gpu_and_oracle(bp, refcuda, name):
    scene = fluid_scene(bp, (14, 14, 14), seed=5, grid_dim=32) if name == "fluid" else small_mixed_scene(bp, seed=5)
    params = bp.make_params(scene)
    out, sdt = _one_substep(bp, refcuda, scene, params)
    h = scene.kernel_radius
    assert out["keys_equal"] and out["order_equal"], "neighbour search differs from the reference's CUDA build"
    e_gpu = float(np.abs(out["gpu"] - out["ref"]).max())
    e_or = float(np.abs(out["oracle"] - out["ref"]).max())
    e_v = float(np.abs(out["gpu_v"] - out["ref_v"]).max())
    assert e_gpu <= 1e-4 * h, f"GB300 solver vs reference CUDA: max |dx| {e_gpu:.3e}"
    assert e_or <= 1e-4 * h, f"oracle vs reference CUDA: max |dx| {e_or:.3e}"
    assert e_v <= 1e-4 * h / sdt, f"GB300 solver vs reference CUDA: max |dv| {e_v:.3e}"


def test_reference_cuda_matches_reference_host_build(bp, refcuda):
    """The same kernels, replayed on the GPU and on the host (OpenMP): the two
    replay drivers launch the same stages in the same order."""
    if refcuda.ref_lib() is None:
        pytest.skip("the reference's host build is unavailable")
    scene = small_mixed_scene(bp, seed=6)
    params = bp.make_params(scene)
    r = refcuda.RefCudaSolver(scene, params)
    c = refcuda.RefSolver(scene, params, threads=1)
    try:
        for s in (r, c):
            s.update(2, DT, 4)
        err = float(np.abs(r.positions() - c.positions()).max())
        assert np.array_equal(r.get(refcuda.F_TO_ORIG), c.get(refcuda.F_TO_ORIG))
    finally:
        r.close()
    assert err <= 2e-4 * scene.kernel_radius, f"CUDA vs host build of the reference: max |dx| {err:.3e}"


def test_reference_cuda_set_state_and_timing(bp, refcuda, gpu):
    """set_state puts a state given in original order back in the identity
    arrangement (where a fresh solver starts: the reference's density sums
    depend on the arrangement); the timed updates advance it like plain
    updates."""
    scene = fluid_scene(bp, (10, 10, 10), seed=7, grid_dim=32)
    params = bp.make_params(scene)
    a = refcuda.RefCudaSolver(scene, params)
    b = refcuda.RefCudaSolver(scene, params)
    try:
        b.update(2, DT, 4)  # moves b away from the initial state and arrangement
        b.set_state(scene.positions, scene.velocities)
        flush = gpu.empty(1 << 20, dtype=gpu.uint8, device="cuda")
        ms = b.time_updates(2, 2, DT, 4, flush.data_ptr(), flush.numel())
        a.update(2, DT, 4)
        a.update(2, DT, 4)
        assert ms > 0.0
        err = float(np.abs(a.positions() - b.positions()).max())
    finally:
        a.close()
        b.close()
    assert err <= 1e-3 * scene.kernel_radius, f"timed updates diverge from plain updates: {err:.3e}"
