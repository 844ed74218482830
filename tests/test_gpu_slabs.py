"""Height slabs (BP_WALK_SLABS): walks over the alias classes that take, per
column, only the quarters of the cells' height a sphere of radius h around
the walker can reach.

They find the same pairs as the full walks and sum them in another order, so
against the oracle they keep the lockstep bar (max |dx| <= 1e-4 h per
substep, identical sorted keys and order), against the other walk variants
they agree to fp32 rounding, and runs with them are bitwise deterministic."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import fluid_scene, small_mixed_scene
from test_gpu_scale import lockstep_from
from test_gpu_solver import DT, assert_parity

pytestmark = pytest.mark.gpu


def slab_params(bp, scene, **kw):
    a = bp.abi
    return bp.make_params(scene, walk_options=a.BP_WALK_NO_STAGING | a.BP_WALK_SLABS, **kw)


@pytest.mark.parametrize("case", ["mixed", "fluid", "aliased", "textbook", "no_split"])
def test_slab_walks_lockstep(bp, gpu, oracle, case):
    a = bp.abi
    if case == "mixed":
        scene = small_mixed_scene(bp, seed=31)
        params = slab_params(bp, scene)
    elif case == "fluid":
        scene = fluid_scene(bp, (14, 14, 14), seed=32, grid_dim=32)
        params = slab_params(bp, scene)
    elif case == "aliased":  # a 1.4 m block on an 8^3 table (1.6 m period): real cells share table cells
        scene = bp.scenes.pbf_scene(14, 8, 14, spacing=0.1, seed=33, box=(2.4, 2.0, 2.4), grid_dim=8)
        params = slab_params(bp, scene)
    elif case == "textbook":
        scene = fluid_scene(bp, (12, 12, 12), seed=34, grid_dim=32)
        params = slab_params(bp, scene, mode=a.BP_MODE_TEXTBOOK, relaxation=600.0, scorr_k=0.001, scorr_dq=0.2,
                             xsph_c=0.01)
    else:
        scene = small_mixed_scene(bp, seed=35)
        params = bp.make_params(scene, walk_options=a.BP_WALK_NO_STAGING | a.BP_WALK_NO_SPLIT | a.BP_WALK_SLABS)
    g = bp.ParticleSolver(scene, params)
    try:
        for _ in range(3):
            g.update(2, DT, 4)
        walks = g.walk_stats(2, DT, 4)
        assert walks["alias_classes"] > 0, walks  # the slab walks ran
        assert_parity(*lockstep_from(bp, oracle, g, scene, params, substeps=6))
    finally:
        g.close()


def test_slab_walks_match_full_walks(bp, gpu):
    """One frame from the same state: slab walks and full walks agree to
    fp32 rounding (the same pairs, summed in another order)."""
    a = bp.abi
    scene = small_mixed_scene(bp, seed=36)
    s1 = bp.ParticleSolver(scene, bp.make_params(scene))
    s2 = bp.ParticleSolver(scene, slab_params(bp, scene))
    try:
        for s in (s1, s2):
            s.update(2, DT, 4)
        assert np.abs(s1.positions() - s2.positions()).max() <= 1e-4 * scene.kernel_radius
        np.testing.assert_array_equal(s1.field(a.BP_FIELD_MAP_TO_ORIGINAL), s2.field(a.BP_FIELD_MAP_TO_ORIGINAL))
    finally:
        s1.close()
        s2.close()


def test_slab_walks_are_deterministic(bp, gpu):
    scene = small_mixed_scene(bp, seed=37)
    outs = []
    for _ in range(2):
        g = bp.ParticleSolver(scene, slab_params(bp, scene))
        for _ in range(5):
            g.update(2, DT, 4)
        outs.append((g.positions(), g.velocities()))
        g.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_slab_walks_mixed_1m_late_lockstep(bp, gpu, oracle):
    """The benchmark's mixed scene (1,146,880 particles) run 200 frames with
    slab walks, then its fluid (planes and fluid) one substep in lockstep."""
    a = bp.abi
    scene = bp.scenes.mixed_phase_1m(seed=0)
    g = bp.ParticleSolver(scene, slab_params(bp, scene, mass_scaling_k=0.0))
    try:
        for _ in range(200):
            g.update(2, DT, 4)
        assert np.isfinite(g.positions()).all() and g.device_errors() == 0
        params = slab_params(bp, scene, mass_scaling_k=0.0, stage_mask=a.BP_STAGE_PLANES | a.BP_STAGE_FLUID)
        g.set_params(params)
        walks = g.walk_stats(1, DT / 2, 4)
        assert walks["alias_classes"] > 0, walks
        assert_parity(*lockstep_from(bp, oracle, g, scene, params, substeps=1))
    finally:
        g.close()
