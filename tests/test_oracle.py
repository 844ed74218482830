"""The oracle (oracle.c) pinned against the reference's own kernels.

Golden fixtures come from the reference kernels compiled for the host
(tests/golden/make_golden.py); the restatement must reproduce them bit for
bit when single-threaded.  Where the reference checkout is present the host
build is also compared live on fresh scenes."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, fluid_scene, small_mixed_scene

import sys

sys.path.insert(0, str(GOLDEN))
from make_golden import scene_from_npz  # noqa: E402

GRID_FIXTURES = ["grid_d32.npz", "grid_d4_alias.npz", "grid_faces_d16.npz", "grid_d512.npz", "grid_single.npz"]
STEP_FIXTURES = ["step_fluid.npz", "step_mixed.npz", "step_mixed_as_shipped.npz", "step_cloth_bending.npz"]


@pytest.mark.parametrize("name", GRID_FIXTURES)
def test_oracle_grid_matches_golden(oracle, name):
    z = np.load(GOLDEN / name)
    pos, cell, D, h = z["positions"], float(z["cell"]), int(z["D"]), float(z["h"])
    cid, scid, spid, cs, ce = oracle.grid_build("oracle", pos, cell, D)
    np.testing.assert_array_equal(cid, z["cell_ids"])
    np.testing.assert_array_equal(scid, z["sorted_cell_ids"])
    np.testing.assert_array_equal(spid, z["sorted_particle_ids"])
    occ = np.nonzero(cs >= 0)[0]
    np.testing.assert_array_equal(occ, z["occupied"])
    np.testing.assert_array_equal(cs[occ], z["cell_start"])
    np.testing.assert_array_equal(ce[occ], z["cell_end"])
    counts = oracle.neighbor_counts("oracle", pos[spid], cell, D, h, cs, ce)
    np.testing.assert_array_equal(counts, z["neighbor_counts"])


def test_grid_sort_is_stable(oracle):
    """Ties keep their current array order (the reference's LSD radix sort)."""
    pos = np.zeros((64, 3), np.float32) + 0.05
    cid, scid, spid, cs, ce = oracle.grid_build("oracle", pos, 0.2, 8)
    np.testing.assert_array_equal(spid, np.arange(64))
    assert (cs >= 0).sum() == 1 and ce[cid[0]] == 64


@pytest.mark.parametrize("name", STEP_FIXTURES)
def test_oracle_step_matches_golden(bp, oracle, name):
    z = np.load(GOLDEN / name)
    scene = scene_from_npz(z, bp.scenes)
    params = bp.make_params(scene)
    params.stage_mask = int(z["stage_mask"])
    o = oracle.OracleSolver(scene, params, threads=1)
    for f in range(int(z["frames"])):
        o.update(2, 1.0 / 60.0, 4)
        if f == 0:
            np.testing.assert_array_equal(o.positions(), z["x1"])
            np.testing.assert_array_equal(o.velocities(), z["v1"])
            np.testing.assert_array_equal(o.get(oracle.F_TO_ORIG), z["to_orig1"])
            np.testing.assert_array_equal(o.get(oracle.F_SORTED_CELL), z["sorted_cell1"])
            np.testing.assert_array_equal(o.get(oracle.F_LAMBDA), z["lambda1"])
            np.testing.assert_array_equal(o.get(oracle.F_DENSITY), z["density1"])
    np.testing.assert_array_equal(o.positions(), z["x"])
    np.testing.assert_array_equal(o.velocities(), z["v"])
    if "rotations" in z:
        np.testing.assert_array_equal(o.get(oracle.F_ROT), z["rotations"])


def test_oracle_moves_things(bp, oracle):
    """The golden mixed scene is not trivially static: every phase moved."""
    z = np.load(GOLDEN / "step_mixed.npz")
    d = np.abs(z["x"] - z["scene_positions"]).max(axis=1)
    ph = z["scene_phases"]
    assert d[ph < 0].max() > 1e-3
    assert d[ph > 0].max() > 1e-3


@pytest.mark.parametrize("threads", [1, 4])
def test_oracle_matches_reference_build_live(bp, oracle, threads):
    if oracle.ref_lib() is None:
        pytest.skip("reference checkout absent: pinned by the golden fixtures instead")
    scene = small_mixed_scene(bp, seed=11)
    params = bp.make_params(scene)
    o = oracle.OracleSolver(scene, params, threads=threads)
    r = oracle.RefSolver(scene, params, threads=threads)
    for _ in range(3):
        o.update(2, 1.0 / 60.0, 4)
        r.update(2, 1.0 / 60.0, 4)
    if threads == 1:
        np.testing.assert_array_equal(o.positions(), r.positions())
    else:  # atomics in a different order: rounding only
        assert np.abs(o.positions() - r.positions()).max() < 1e-4 * scene.kernel_radius


def test_oracle_picking_matches_reference(bp, oracle):
    if oracle.ref_lib() is None:
        pytest.skip("reference checkout absent")
    scene = fluid_scene(bp, (6, 6, 6), seed=2, grid_dim=16)
    params = bp.make_params(scene)
    o = oracle.OracleSolver(scene, params)
    r = oracle.RefSolver(scene, params)
    pp = np.array([0.5, 1.5, 0.5], np.float32)
    pv = np.array([1.0, 0.0, 0.0], np.float32)
    for _ in range(2):
        o.update(2, 1 / 60, 3, picked=7, picked_position=pp, picked_velocity=pv)
        r.update(2, 1 / 60, 3, picked=7, picked_position=pp, picked_velocity=pv)
    np.testing.assert_array_equal(o.positions(), r.positions())
    np.testing.assert_array_equal(o.velocities(), r.velocities())


def test_reference_params_match_product_literals(bp, oracle):
    """oracle.reference_params (used by the CPU reference arm, which loads no
    product code) gives exactly what make_params gives."""
    for scene in (fluid_scene(bp, (4, 4, 4), seed=1), small_mixed_scene(bp, seed=1)):
        a, b = bp.make_params(scene), oracle.reference_params(scene)
        assert bytes(a) == bytes(b)
        a, b = bp.make_params(scene, mass_scaling_k=0.0), oracle.reference_params(scene, mass_scaling_k=0.0)
        assert bytes(a) == bytes(b)


def test_reference_mass_scaling_parameter(bp, oracle):
    """The reference replay takes the mass-scaling k as a parameter (the
    literal 2 at its call site): k = 0 gives what the oracle gives at k = 0."""
    if oracle.ref_lib() is None:
        pytest.skip("reference sources absent")
    scene = small_mixed_scene(bp, seed=12)
    params = bp.make_params(scene, mass_scaling_k=0.0)
    o = oracle.OracleSolver(scene, params)
    r = oracle.RefSolver(scene, params)
    o.update(2, 1.0 / 60.0, 4)
    r.update(2, 1.0 / 60.0, 4)
    np.testing.assert_array_equal(o.positions(), r.positions())
    np.testing.assert_array_equal(o.get(oracle.F_INVSCALED), r.get(oracle.F_INVSCALED))


def test_reference_cuda_build_exports(oracle):
    """The reference's sm_103a build loads without a GPU and exports the
    replay driver's entry points (its compute calls need the GPU)."""
    if oracle.ref_source() is None:
        pytest.skip("reference sources absent")
    import ctypes

    lib = ctypes.CDLL(str(oracle.build_ref_cuda()))
    for name in ("refcu_create", "refcu_destroy", "refcu_update", "refcu_time_updates", "refcu_set_state",
                 "refcu_get", "refcu_error"):
        assert hasattr(lib, name), name


def test_fp64_oracle_tracks_fp32(bp, oracle):
    """The FP64 host oracle is the same source in double: it builds the same
    grid (the cell hash stays float arithmetic) and its state stays within
    fp32 rounding of the fp32 oracle's over a few frames."""
    scene = fluid_scene(bp, (10, 10, 10), seed=1, grid_dim=32)
    params = oracle.reference_params(scene)
    a = oracle.OracleSolver(scene, params)
    b = oracle.OracleSolver(scene, params, precision=64)
    for _ in range(3):
        a.update(2, 1.0 / 60.0, 4)
        b.update(2, 1.0 / 60.0, 4)
    assert b.positions().dtype == np.float64
    np.testing.assert_array_equal(a.get(oracle.F_TO_ORIG), b.get(oracle.F_TO_ORIG))
    assert np.abs(a.positions() - b.positions()).max() < 1e-5


def test_fp64_oracle_parameter_overrides(bp, oracle):
    """Wind and stiffness set in double change the rollout as the same values
    set through the parameters do."""
    import copy

    abi = bp.abi
    scene = bp.scenes.flag_scene(n=8, seed=2)
    stages = abi.BP_STAGE_PLANES | abi.BP_STAGE_WIND | abi.BP_STAGE_DISTANCE | abi.BP_STAGE_IMMOVABLE
    params = oracle.reference_params(scene, mode=abi.BP_MODE_TEXTBOOK, stage_mask=stages,
                                     wind_velocity=(4.0, 0.0, 0.0), wind_drag=1.0, wind_lift=0.3, mass_scaling_k=0.0)
    p2 = copy.copy(params)
    p2.wind_velocity[1] = 2.0
    sc2 = copy.deepcopy(scene)
    sc2.distance_params[:, 1] *= 0.5
    a = oracle.OracleSolver(sc2, p2, precision=64)
    b = oracle.OracleSolver(scene, params, precision=64)
    b.set_wind(np.array([4.0, 2.0, 0.0]))
    dp = scene.distance_params.astype(np.float64)
    dp[:, 1] *= 0.5
    b.set_distance_params(dp)
    for s in (a, b):
        for _ in range(3):
            s.update(2, 1.0 / 60.0, 4)
    np.testing.assert_array_equal(a.positions(), b.positions())
