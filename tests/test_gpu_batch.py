"""Batched ensembles on the GPU through the C ABI.

A batch steps many scenes in one launch per stage through a segmented hash
grid.  Each scene's particles must follow exactly (bit for bit) the trajectory
that a solver of that scene alone gives, so the single-scene parity against the
oracle carries over to every member of a batch."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import cloth_bending_scene, small_mixed_scene

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def members(bp):
    sc = bp.scenes
    scenes = [
        sc.ensemble_member(300, seed=1),
        sc.ensemble_member(2000, seed=2, rest_scale=0.85, gravity=13.0),
        small_mixed_scene(bp, seed=3),
        sc.ensemble_member(900, seed=4, rest_scale=1.15, gravity=6.0),
        cloth_bending_scene(bp, seed=5, n=8),  # dihedral bending quads, offset in the batch
    ]
    return scenes


@pytest.mark.parametrize("walk", [0, 1])
def test_batch_members_match_single_scene_solvers(bp, gpu, walk):
    scenes = members(bp)
    params = [bp.make_params(s, walk_options=walk * bp.abi.BP_WALK_NO_STAGING) for s in scenes]
    batch = bp.BatchSolver(scenes, params)
    singles = [bp.ParticleSolver(s, p) for s, p in zip(scenes, params)]
    for _ in range(5):
        batch.update(2, DT, 4)
        for g in singles:
            g.update(2, DT, 4)
    x, v = batch.positions(), batch.velocities()
    for k, g in enumerate(singles):
        first, count = batch.ranges[k]
        assert count == scenes[k].num_particles
        np.testing.assert_array_equal(x[first:first + count], g.positions(), err_msg=f"scene {k}")
        np.testing.assert_array_equal(v[first:first + count], g.velocities(), err_msg=f"scene {k}")
        g.close()
    assert batch.device_errors() == 0
    batch.close()


def test_batch_scene_ranges_and_step(bp, gpu):
    scenes = [bp.scenes.ensemble_member(n, seed=n) for n in (150, 700, 64)]
    batch = bp.BatchSolver(scenes)
    firsts = [r[0] for r in batch.ranges]
    counts = [r[1] for r in batch.ranges]
    assert firsts == list(np.cumsum([0] + counts[:-1]))
    assert counts == [s.num_particles for s in scenes]
    x0 = batch.positions()
    batch.step(DT, 2, 4)
    x1 = batch.positions()
    assert np.isfinite(x1).all() and not np.array_equal(x0, x1)
    # each scene stays inside its own walls
    for k, s in enumerate(scenes):
        xs = batch.scene_positions(k)
        hi = s.planes[:, :3].max(axis=0)
        assert (xs >= -1e-3).all()
        assert (xs[:, [0, 2]] <= hi[[0, 2]] + 1e-3).all()
    batch.close()


@pytest.mark.parametrize("grid_dim", [16, 64, 128])
def test_solid_cell_masks_keep_collision_bits(bp, gpu, grid_dim):
    """A single-scene solver lets fluid skip its walk over the solids where
    no solid is stored in its 27 cells (a per-substep cell mask); a batch
    walks them all.  The mixed scene sits across z cell 63/64 (x + 50000 over
    the cell size, masked), so the mask's dilation wraps rows (64) and crosses
    words (128); bodies fall onto the fluid within the frames run."""
    s = small_mixed_scene(bp, seed=7, grid_dim=grid_dim)
    dz = 9.3
    s.positions[:, 2] += dz
    s.planes[:, 2] += dz
    p = bp.make_params(s)
    single = bp.ParticleSolver(s, p)
    batch = bp.BatchSolver([s], [p])
    for _ in range(20):
        single.update(2, DT, 4)
        batch.update(2, DT, 4)
    np.testing.assert_array_equal(batch.positions(), single.positions())
    np.testing.assert_array_equal(batch.velocities(), single.velocities())
    assert single.device_errors() == 0 and batch.device_errors() == 0
    single.close()
    batch.close()
