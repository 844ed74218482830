"""The solver step on the GPU through the C ABI against the oracle.

Parity bar: from identical inputs, one substep of the GPU solver and of the
oracle (the reference's step restated, pinned bit-exact to the reference's
own kernels) agree to max |x_gpu - x_oracle| <= 1e-4 * h, velocities to
1e-4 * h / dt; the neighbour search inside the step (cell keys, stable sorted
order) is identical.  The GPU sums pair terms in a different order than the
reference's atomics, so fp32 rounding differs; nothing else may."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, cloth_bending_scene, fluid_scene, small_mixed_scene

import sys

sys.path.insert(0, str(GOLDEN))
from make_golden import scene_from_npz  # noqa: E402

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def gpu_state(bp, s):
    abi = bp.abi
    X = s.field(abi.BP_FIELD_POSITIONS)
    V = s.field(abi.BP_FIELD_VELOCITIES)
    to_orig = s.field(abi.BP_FIELD_MAP_TO_ORIGINAL)
    rot = s.field(abi.BP_FIELD_RIGID_ROTATIONS) if len(s.scene.rigid_ranges) else None
    return X[:, :3].copy(), V[:, :3].copy(), to_orig, rot


def lockstep(bp, oracle, scene, params, substeps=6, iterations=4, sub_per_call=1):
    """Runs GPU and oracle substep by substep, re-synchronising the oracle on
    the GPU state before each one; returns per-substep max errors."""
    g = bp.ParticleSolver(scene, params)
    o = oracle.OracleSolver(scene, params)
    h = scene.kernel_radius
    sdt = DT / 2
    errs = []
    for k in range(substeps):
        x, v, to_orig, rot = gpu_state(bp, g)
        o.adopt(x, v, to_orig, rot)
        g.update(sub_per_call, sdt * sub_per_call, iterations)
        o.update(sub_per_call, sdt * sub_per_call, iterations)
        ex = np.abs(g.positions() - o.positions()).max()
        ev = np.abs(g.velocities() - o.velocities()).max()
        keys_equal = np.array_equal(g.field(bp.abi.BP_FIELD_SORTED_CELL_IDS), o.get(oracle.F_SORTED_CELL))
        order_equal = np.array_equal(g.field(bp.abi.BP_FIELD_MAP_TO_ORIGINAL), o.get(oracle.F_TO_ORIG))
        errs.append((ex, ev, keys_equal, order_equal))
    g.close()
    return errs, h, sdt


def assert_parity(errs, h, sdt):
    for k, (ex, ev, keys_equal, order_equal) in enumerate(errs):
        assert keys_equal and order_equal, f"substep {k}: neighbour search differs"
        assert ex <= 1e-4 * h, f"substep {k}: max position error {ex:.3e} > {1e-4 * h:.3e}"
        assert ev <= 1e-4 * h / sdt, f"substep {k}: max velocity error {ev:.3e}"


def test_fluid_substep_parity(bp, gpu, oracle):
    scene = fluid_scene(bp, (14, 14, 14), seed=1, grid_dim=32)
    errs, h, sdt = lockstep(bp, oracle, scene, bp.make_params(scene), substeps=8)
    assert_parity(errs, h, sdt)


def test_mixed_substep_parity(bp, gpu, oracle):
    scene = small_mixed_scene(bp, seed=2)
    errs, h, sdt = lockstep(bp, oracle, scene, bp.make_params(scene), substeps=8)
    assert_parity(errs, h, sdt)


@pytest.mark.parametrize("iterations", [1, 2, 3])
def test_mixed_parity_iteration_counts(bp, gpu, oracle, iterations):
    scene = small_mixed_scene(bp, seed=3)
    errs, h, sdt = lockstep(bp, oracle, scene, bp.make_params(scene), substeps=3, iterations=iterations)
    assert_parity(errs, h, sdt)


@pytest.mark.parametrize("mask_name", ["as_shipped", "no_akinci", "fluid_only", "constraints_only"])
def test_stage_subsets_parity(bp, gpu, oracle, mask_name):
    a = bp.abi
    masks = {
        "as_shipped": a.BP_STAGE_REFERENCE_AS_SHIPPED | a.BP_STAGE_FLUID,
        "no_akinci": a.BP_STAGE_ALL & ~a.BP_STAGE_AKINCI,   # s_corr on, no C clamp
        "fluid_only": a.BP_STAGE_PLANES | a.BP_STAGE_FLUID,
        "constraints_only": a.BP_STAGE_PLANES | a.BP_STAGE_DISTANCE | a.BP_STAGE_WIND | a.BP_STAGE_SHAPE_MATCHING
        | a.BP_STAGE_IMMOVABLE | a.BP_STAGE_PARTICLE_COLLISION,
    }
    scene = small_mixed_scene(bp, seed=4)
    params = bp.make_params(scene, stage_mask=masks[mask_name])
    errs, h, sdt = lockstep(bp, oracle, scene, params, substeps=4)
    assert_parity(errs, h, sdt)


def test_large_rigid_bodies_parity(bp, gpu, oracle):
    """Shape matching of bodies far beyond the reference kernel's 64-particle
    limit (a 512-particle cube and a 1000-particle slab, as in the mixed and
    shape-matching configurations), falling onto the floor and onto each other
    with particle collisions, in lockstep with the oracle."""
    sc = bp.scenes
    s = sc.Scene(name="big_rigid")
    s.particle_radius, s.kernel_radius, s.cell_size, s.grid_dim, s.rest_density = 0.05, 0.2, 0.2, 32, 1000.0
    sc.box_planes(s, (0, 0, 0), (3.0, 4.0, 3.0))
    s.add_rigid_box((8, 8, 8), (0.6, 0.3, 0.6), (0.1, 0.1, 0.1), 1.0)
    s.add_rigid_box((10, 4, 25), (0.3, 1.4, 0.2), (0.1, 0.1, 0.1), 1.0)
    rng = np.random.default_rng(17)
    s.velocities = np.repeat(rng.uniform(-1.0, 1.0, (1, 3)), s.num_particles, axis=0).astype(np.float32)
    s.velocities[:512] += rng.uniform(-0.2, 0.2, (512, 3)).astype(np.float32)  # spin the cube
    assert [r1 - r0 for r0, r1 in s.rigid_ranges] == [512, 1000]
    assert_parity(*lockstep(bp, oracle, s, bp.make_params(s), substeps=6))


def test_dihedral_bending_parity(bp, gpu, oracle):
    """Dihedral bending (kernel/bending.cuh) on a sagging cloth with its
    stretch, shear and skip-one pairs, self-collisions and pinned corners."""
    scene = cloth_bending_scene(bp, seed=3)
    assert len(scene.bendings) == 121
    assert_parity(*lockstep(bp, oracle, scene, bp.make_params(scene), substeps=6))
    # the stage does something: without it the cloth ends elsewhere
    a = bp.ParticleSolver(scene, bp.make_params(scene))
    b = bp.ParticleSolver(scene, bp.make_params(scene, stage_mask=bp.abi.BP_STAGE_ALL & ~bp.abi.BP_STAGE_BENDING))
    for s in (a, b):
        for _ in range(5):
            s.update(2, DT, 4)
    assert np.abs(a.positions() - b.positions()).max() > 1e-3
    a.close()
    b.close()


def test_textbook_mode_parity(bp, gpu, oracle):
    # s_corr k = 0.001: with m = 1 kg and rho0 = 1000 kg/m^3 the paper's k = 0.1
    # outweighs lambda ~50x and the block explodes (on the oracle as well)
    scene = fluid_scene(bp, (12, 12, 12), seed=5, grid_dim=32)
    params = bp.make_params(scene, mode=bp.abi.BP_MODE_TEXTBOOK, relaxation=600.0, scorr_k=0.001, scorr_dq=0.2,
                            xsph_c=0.01)
    errs, h, sdt = lockstep(bp, oracle, scene, params, substeps=4)
    assert_parity(errs, h, sdt)


def test_two_substeps_per_call_parity(bp, gpu, oracle):
    scene = small_mixed_scene(bp, seed=7)
    errs, h, sdt = lockstep(bp, oracle, scene, bp.make_params(scene), substeps=3, sub_per_call=2)
    assert_parity(errs, h, sdt)


@pytest.mark.parametrize("name", ["step_fluid.npz", "step_mixed.npz", "step_mixed_as_shipped.npz",
                                  "step_cloth_bending.npz"])
def test_first_frame_matches_reference_golden(bp, gpu, name):
    """One frame from the fixture scene against the reference's own kernels."""
    z = np.load(GOLDEN / name)
    scene = scene_from_npz(z, bp.scenes)
    params = bp.make_params(scene)
    params.stage_mask = int(z["stage_mask"])
    g = bp.ParticleSolver(scene, params)
    g.update(2, DT, 4)
    h = scene.kernel_radius
    # The self-colliding cloth (144 particles all in contact range of their
    # lattice neighbours, plus bending and stretch) amplifies rounding over the
    # frame's 8 constraint passes: 4.2e-5 measured there, so it gets 4e-4 h.
    tol = 4e-4 if name == "step_cloth_bending.npz" else 2e-4
    np.testing.assert_array_less(np.abs(g.positions() - z["x1"]).max(), tol * h)
    np.testing.assert_array_equal(g.field(bp.abi.BP_FIELD_MAP_TO_ORIGINAL), z["to_orig1"])
    np.testing.assert_array_equal(g.field(bp.abi.BP_FIELD_SORTED_CELL_IDS), z["sorted_cell1"])
    g.close()


def test_density_statistics_100_frames(bp, gpu, oracle):
    """Free-running for 100 frames, the fluid's density error statistics agree
    with the oracle's (trajectories decorrelate; the statistics must not)."""
    scene = fluid_scene(bp, (10, 10, 10), seed=8, grid_dim=32)
    params = bp.make_params(scene)
    g = bp.ParticleSolver(scene, params)
    o = oracle.OracleSolver(scene, params, threads=4)
    stats_g, stats_o = [], []
    for f in range(100):
        g.update(2, DT, 4)
        o.update(2, DT, 4)
        if f >= 50:
            rg = g.field(bp.abi.BP_FIELD_DENSITIES)
            ro = o.get(oracle.F_DENSITY)
            stats_g.append(rg.mean())
            stats_o.append(ro.mean())
    mg, mo = float(np.mean(stats_g)), float(np.mean(stats_o))
    assert abs(mg - mo) / mo < 0.02, (mg, mo)
    assert np.isfinite(g.positions()).all()
    g.close()


def test_runs_are_bitwise_deterministic(bp, gpu):
    scene = small_mixed_scene(bp, seed=9)
    outs = []
    for _ in range(2):
        g = bp.ParticleSolver(scene, bp.make_params(scene))
        for _ in range(5):
            g.update(2, DT, 4)
        outs.append((g.positions(), g.velocities()))
        g.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("skin", [0.3, 0.1, 0.02, 0.001])
def test_verlet_lists_are_bit_identical_to_cell_walks(bp, gpu, skin):
    """The per-substep Verlet lists (any skin, including one so small that
    the displacement guard sends most walks back to the cells mid-substep)
    give exactly the results of walking the 27 cells."""
    scene = small_mixed_scene(bp, seed=13)
    outs = []
    for s in (0.0, skin):
        g = bp.ParticleSolver(scene, bp.make_params(scene, neighbor_skin=s))
        assert g.params.neighbor_skin == np.float32(s)
        walks = g.walk_stats(2, DT, 4)  # a real update
        if s >= 0.1:
            assert walks["listed"] > walks["cells_displaced"], walks
        if s == 0.001:
            assert walks["cells_displaced"] > 0, walks
        for _ in range(3):
            g.update(2, DT, 4)
        outs.append((g.positions(), g.velocities()))
        g.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("skin", [0.0, 0.1])
@pytest.mark.parametrize("walk", ["no_staging", "no_split", "no_lists", "none"])
def test_walk_variants_are_bit_identical(bp, gpu, walk, skin):
    """Staging each block's neighbourhood in shared memory, testing
    candidates in chunks before the pair terms and the post passes'
    neighbour lists change nothing: every walk variant gives the default
    walk's bits."""
    abi = bp.abi
    options = {"no_staging": abi.BP_WALK_NO_STAGING, "no_split": abi.BP_WALK_NO_SPLIT,
               "no_lists": abi.BP_WALK_NO_LISTS,
               "none": abi.BP_WALK_NO_STAGING | abi.BP_WALK_NO_SPLIT | abi.BP_WALK_NO_LISTS}[walk]
    scene = small_mixed_scene(bp, seed=14)
    outs = []
    for w in (0, options):
        g = bp.ParticleSolver(scene, bp.make_params(scene, walk_options=w, neighbor_skin=skin))
        for _ in range(4):
            g.update(2, DT, 4)
        outs.append((g.positions(), g.velocities()))
        g.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("skin", [0.0, 0.1])
@pytest.mark.parametrize("walk", ["split", "no_split"])
def test_lists_overflowing_their_capacity_are_bit_identical(bp, gpu, walk, skin):
    """A block packed at half spacing holds about 270 neighbours within h
    per particle, past the 192 entries a list takes (and the 256 of a Verlet
    list): those particles walk their cells, the others read lists, and the
    bits equal walks everywhere."""
    abi = bp.abi
    base = abi.BP_WALK_NO_STAGING | (abi.BP_WALK_NO_SPLIT if walk == "no_split" else 0)
    scene = fluid_scene(bp, (12, 12, 12), seed=31, grid_dim=32)
    x = scene.positions.copy()
    c = x.mean(axis=0)
    dense = np.all(np.abs(x - c) < 0.35, axis=1)
    x[dense] = c + (x[dense] - c) * np.float32(0.5)
    scene.positions = x.astype(np.float32)
    assert dense.sum() > 200
    outs = []
    for w, sk in ((base, skin), (base | abi.BP_WALK_NO_LISTS, 0.0)):
        g = bp.ParticleSolver(scene, bp.make_params(scene, walk_options=w, neighbor_skin=sk))
        for _ in range(3):
            g.update(2, DT, 4)
        outs.append((g.positions(), g.velocities()))
        g.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("mode", ["reference", "textbook"])
def test_overflowing_class_position_lists_are_bit_identical(bp, gpu, mode):
    """The overflow case on an 8^3 table, where the walks take the alias
    classes and the lists hold class positions: particles past the list
    capacity walk their cells with sorted indices, the rest read class
    positions, and the bits equal walks everywhere."""
    abi = bp.abi
    m = abi.BP_MODE_TEXTBOOK if mode == "textbook" else abi.BP_MODE_REFERENCE
    scene = fluid_scene(bp, (20, 8, 20), seed=37, grid_dim=8, box=(2.5, 3.0, 2.5))
    x = scene.positions.copy()
    c = x.mean(axis=0)
    dense = np.all(np.abs(x - c) < 0.35, axis=1)
    x[dense] = c + (x[dense] - c) * np.float32(0.5)
    scene.positions = x.astype(np.float32)
    assert dense.sum() > 200
    outs = []
    for w in (abi.BP_WALK_NO_STAGING, abi.BP_WALK_NO_STAGING | abi.BP_WALK_NO_LISTS):
        g = bp.ParticleSolver(scene, bp.make_params(scene, mode=m, walk_options=w))
        walks = g.walk_stats(1, DT / 2, 4)  # a real update
        assert walks["alias_classes"] > 0, walks
        for _ in range(3):
            g.update(2, DT, 4)
        outs.append((g.positions(), g.velocities()))
        g.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("walk", ["split", "no_split", "staging", "textbook"])
def test_alias_classes_are_bit_identical(bp, gpu, walk):
    """An 8^3 table over a 3 x 4 x 3 m box: every table cell holds up to
    eight real cells.  Walks restricted to the walked real cell's alias class
    give the bits of walks over whole table cells (with the threads in class
    order and the position pass's lists in class positions)."""
    abi = bp.abi
    base = {"split": abi.BP_WALK_NO_STAGING, "no_split": abi.BP_WALK_NO_STAGING | abi.BP_WALK_NO_SPLIT,
            "staging": 0, "textbook": abi.BP_WALK_NO_STAGING}[walk]
    mode = abi.BP_MODE_TEXTBOOK if walk == "textbook" else abi.BP_MODE_REFERENCE
    scene = small_mixed_scene(bp, seed=15, fluid=(20, 8, 20), grid_dim=8)
    outs = []
    for w in (base, base | abi.BP_WALK_NO_ALIAS_CLASSES):
        g = bp.ParticleSolver(scene, bp.make_params(scene, mode=mode, walk_options=w))
        walks = g.walk_stats(2, DT, 4)  # a real update
        if w & abi.BP_WALK_NO_ALIAS_CLASSES:
            assert walks["alias_classes"] == 0
        elif walk != "staging":
            assert walks["alias_classes"] > walks["cells_no_list"] // 2, walks
        for _ in range(5):
            g.update(2, DT, 4)
        outs.append((g.positions(), g.velocities()))
        g.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_split_walks_match_one_thread_walks_on_aliased_grid(bp, gpu):
    """Split walks (chunks of candidates tested before the pair terms)
    against fused walks on the 8^3 table, where the walks take the alias
    classes and the lists hold class positions: same bits."""
    abi = bp.abi
    scene = small_mixed_scene(bp, seed=17, fluid=(20, 8, 20), grid_dim=8)
    outs = []
    for w in (abi.BP_WALK_NO_STAGING, abi.BP_WALK_NO_STAGING | abi.BP_WALK_NO_SPLIT):
        g = bp.ParticleSolver(scene, bp.make_params(scene, walk_options=w))
        walks = g.walk_stats(2, DT, 4)  # a real update
        assert walks["alias_classes"] > walks["cells_no_list"] // 2, walks
        for _ in range(5):
            g.update(2, DT, 4)
        outs.append((g.positions(), g.velocities()))
        g.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("case", ["sorted", "classes", "no_classes", "textbook"])
def test_walk_planes_are_bit_identical(bp, gpu, case):
    """The walks that record the lambda pass's and post pass A's lists read
    their candidates from the walk planes (x, y, z and phase in arrays of
    their own, four candidates per three loads, paired fp32 arithmetic) and
    append each chunk's hits a record at a time: the same lists and bits as
    walks over the position records, with the planes in sorted order
    (classes gated off, or none), in class order (8^3 table) and in textbook
    mode."""
    abi = bp.abi
    base = abi.BP_WALK_NO_STAGING | (abi.BP_WALK_NO_ALIAS_CLASSES if case == "no_classes" else 0)
    mode = abi.BP_MODE_TEXTBOOK if case == "textbook" else abi.BP_MODE_REFERENCE
    aliased = case in ("classes", "textbook")
    scene = small_mixed_scene(bp, seed=19, fluid=(20, 8, 20) if aliased else (10, 10, 10),
                              grid_dim=8 if aliased else 32)
    outs = []
    for w in (base, base | abi.BP_WALK_NO_PLANES):
        g = bp.ParticleSolver(scene, bp.make_params(scene, mode=mode, walk_options=w))
        walks = g.walk_stats(2, DT, 4)  # a real update
        if aliased:
            assert walks["alias_classes"] > walks["cells_no_list"] // 2, walks
        else:
            assert walks["alias_classes"] == 0, walks
        for _ in range(5):
            g.update(2, DT, 4)
        outs.append((g.positions(), g.velocities()))
        g.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_alias_classes_parity_on_aliased_grid(bp, gpu, oracle):
    scene = small_mixed_scene(bp, seed=16, fluid=(20, 8, 20), grid_dim=8)
    assert_parity(*lockstep(bp, oracle, scene, bp.make_params(scene), substeps=4))


def test_alias_classes_fall_back_past_the_reach(bp, gpu):
    """Particles placed exactly one table period (8 cells, 1.6 m) below the
    floor: the plane stabilisation lifts them into the table cell they were
    hashed to, next to the fluid, but their hash-time class is the other one.
    They moved further than the reach, so the walks take whole table cells
    and find them; the bits equal those of class-free walks."""
    abi = bp.abi
    scene = fluid_scene(bp, (20, 6, 20), seed=23, grid_dim=8, box=(2.5, 3.0, 2.5))
    x = scene.positions.copy()
    low = np.argsort(x[:, 1])[:50]
    x[low, 1] -= np.float32(8 * scene.cell_size)
    scene.positions = x
    outs = []
    for w in (abi.BP_WALK_NO_STAGING, abi.BP_WALK_NO_STAGING | abi.BP_WALK_NO_ALIAS_CLASSES):
        g = bp.ParticleSolver(scene, bp.make_params(scene, walk_options=w))
        first = g.walk_stats(1, DT / 2, 4)  # a real update: the lift
        assert first["alias_classes"] == 0, first
        xs = [g.positions()]
        later = g.walk_stats(1, DT / 2, 4)  # nothing moves that far now
        if not w & abi.BP_WALK_NO_ALIAS_CLASSES:
            assert later["alias_classes"] > 0, later
        for _ in range(2):
            g.update(2, DT, 4)
        outs.append((xs[0], g.positions(), g.velocities()))
        g.close()
    assert np.all(outs[0][0][low, 1] > 0.0)  # lifted onto the floor
    for a, b in zip(outs[0], outs[1]):
        np.testing.assert_array_equal(a, b)


def test_autotune_keeps_state_and_results(bp, gpu):
    """The autotuner's trial updates leave the state as it was, and the walk
    variant and launch shape it keeps give the same bits as the defaults."""
    abi = bp.abi
    scene = small_mixed_scene(bp, seed=21)
    a = bp.ParticleSolver(scene, bp.make_params(scene))
    b = bp.ParticleSolver(scene, bp.make_params(scene))
    for s in (a, b):
        s.update(2, DT, 4)
    x0 = a.positions()
    opt, ms = a.autotune(2, DT, 4)
    np.testing.assert_array_equal(a.positions(), x0)
    assert 0 <= opt <= (abi.BP_WALK_NO_SPLIT | abi.BP_WALK_NO_LISTS | abi.BP_WALK_NO_STAGING |
                        abi.BP_WALK_NO_FUSION | abi.BP_WALK_NO_CONTACT_CULLING)
    assert not opt & abi.BP_WALK_NO_ALIAS_CLASSES
    assert len(ms) == 13
    assert all(t > 0 for t in ms[:8]) and ms[11] > 0 and ms[12] > 0  # the scene has contacts
    assert a.params.scan_block in (0, 64, 128, 256) and a.params.scan_persistent in (0, 1)
    assert all(t > 0 for t in ms[8:11]) == bool(opt & abi.BP_WALK_NO_STAGING)
    for s in (a, b):
        for _ in range(3):
            s.update(2, DT, 4)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.velocities(), b.velocities())
    a.close()
    b.close()


@pytest.mark.parametrize("shape", [(128, 0), (64, 0), (256, 1), (128, 1)])
def test_scan_launch_shapes_are_bit_identical(bp, gpu, shape):
    """Unstaged scans with other CTA sizes, or persistent CTAs striding over
    the tiles, give the same bits as the default launch."""
    abi = bp.abi
    scene = small_mixed_scene(bp, seed=23)
    base = bp.make_params(scene, walk_options=abi.BP_WALK_NO_STAGING)
    other = bp.make_params(scene, walk_options=abi.BP_WALK_NO_STAGING, scan_block=shape[0],
                           scan_persistent=shape[1])
    outs = []
    for p in (base, other):
        g = bp.ParticleSolver(scene, p)
        for _ in range(4):
            g.update(2, DT, 4)
        outs.append((g.positions(), g.velocities()))
        g.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_iteration_fusion_is_bit_identical(bp, gpu):
    """Plane collision and the final commit fused into the reorder and the
    position pass's epilogue (the default) or run as launches of their own
    (BP_WALK_NO_FUSION): the same bits, on a fluid scene with planes and on
    the mixed scene (whose constraint stages leave only the first fusion)."""
    abi = bp.abi
    for scene in (fluid_scene(bp, seed=24), small_mixed_scene(bp, seed=24)):
        outs = []
        for opt in (0, abi.BP_WALK_NO_FUSION):
            g = bp.ParticleSolver(scene, bp.make_params(scene, walk_options=opt))
            for _ in range(4):
                g.update(2, DT, 4)
            outs.append((g.positions(), g.velocities()))
            g.close()
        np.testing.assert_array_equal(outs[0][0], outs[1][0])
        np.testing.assert_array_equal(outs[0][1], outs[1][1])


def contact_scene(bp, seed=0):
    """Grains, two rigid boxes and a rope over a fluid pool, with random
    velocities: contacts between every pair of phases."""
    sc = bp.scenes
    rng = np.random.default_rng(seed)
    s = sc.Scene(name="contacts")
    s.particle_radius, s.kernel_radius, s.cell_size, s.grid_dim, s.rest_density = 0.05, 0.2, 0.2, 16, 1000.0
    sc.box_planes(s, (0, 0, 0), (1.6, 3.0, 1.6))
    s.add_fluid_block((12, 4, 12), (0.1, 0.05, 0.1), (0.1, 0.1, 0.1), 1.0, jitter=0.002, rng=rng)
    s.add_granulars_block((5, 5, 5), (0.4, 0.5, 0.4), (0.095, 0.095, 0.095), 1.0)
    s.add_rigid_box((3, 3, 3), (0.9, 0.7, 0.9), (0.1, 0.1, 0.1), 1.0)
    s.add_rigid_box((4, 2, 3), (0.2, 1.1, 0.9), (0.1, 0.1, 0.1), 1.0)
    s.add_rope((0.1, 1.4, 0.2), (1.4, 1.4, 1.3), 16, 0.5)
    s.velocities = rng.uniform(-0.5, 0.5, (s.num_particles, 3)).astype(np.float32)
    return s


@pytest.mark.parametrize("walk", [0, "NO_STAGING", "NO_SPLIT", "VERLET"])
def test_contact_culling_is_bit_identical(bp, gpu, walk):
    """Contact walks over only the cells a partner can be stored in against
    the full 27-cell walks (BP_WALK_NO_CONTACT_CULLING): the same bits, on a
    scene with contacts between every pair of phases (mostly fluid: only the
    fluid walkers cull), the mixed scene and grains alone (all solids: the
    solids cull too), also with Verlet lists (whose entries a culled walk may
    test instead of its cells)."""
    abi = bp.abi
    skin = 0.3 if walk == "VERLET" else 0.0
    wo = 0 if walk in (0, "VERLET") else getattr(abi, "BP_WALK_" + walk)
    grains = bp.scenes.Scene(name="grains")
    grains.particle_radius, grains.kernel_radius, grains.cell_size, grains.grid_dim = 0.05, 0.2, 0.2, 16
    bp.scenes.box_planes(grains, (0, 0, 0), (1.6, 3.0, 1.6))
    grains.add_granulars_block((6, 6, 6), (0.3, 0.2, 0.3), (0.09, 0.09, 0.09), 1.0)
    for scene in (contact_scene(bp, seed=5), small_mixed_scene(bp, seed=25), grains):
        outs = []
        for opt in (wo, wo | abi.BP_WALK_NO_CONTACT_CULLING):
            g = bp.ParticleSolver(scene, bp.make_params(scene, walk_options=opt, neighbor_skin=skin))
            for _ in range(6):
                g.update(2, DT, 4)
            outs.append((g.positions(), g.velocities()))
            g.close()
        np.testing.assert_array_equal(outs[0][0], outs[1][0])
        np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_snapshot_resume_is_bit_identical(bp, gpu):
    """Checkpoint / resume: a solver loaded from a snapshot continues exactly
    as the one that was never interrupted (sorted order, rigid rotations and
    all), and a snapshot of another scene is refused."""
    abi = bp.abi
    scene = small_mixed_scene(bp, seed=19)
    p = bp.make_params(scene)
    a = bp.ParticleSolver(scene, p)
    for _ in range(4):
        a.update(2, DT, 4)
    snap = a.snapshot()
    for _ in range(3):
        a.update(2, DT, 4)
    b = bp.ParticleSolver(scene, p)
    b.update(2, DT, 4)  # some other state first
    b.restore(snap)
    for _ in range(3):
        b.update(2, DT, 4)
    for f in (abi.BP_FIELD_POSITIONS, abi.BP_FIELD_VELOCITIES, abi.BP_FIELD_MAP_TO_ORIGINAL,
              abi.BP_FIELD_RIGID_ROTATIONS, abi.BP_FIELD_DENSITIES):
        np.testing.assert_array_equal(a.field(f), b.field(f), err_msg=f"field {f}")
    other = fluid_scene(bp, (4, 4, 4), seed=1, grid_dim=16)
    c = bp.ParticleSolver(other, bp.make_params(other))
    with pytest.raises(bp.BrassPanError):
        c.restore(snap)
    with pytest.raises(bp.BrassPanError):
        c.restore(b"not a snapshot at all, just some bytes of text")
    for s in (a, b, c):
        s.close()


def test_graph_replay_equals_recapture(bp, gpu):
    scene = small_mixed_scene(bp, seed=10)
    p = bp.make_params(scene)
    a = bp.ParticleSolver(scene, p)
    b = bp.ParticleSolver(scene, p)
    for _ in range(4):
        a.update(2, DT, 4)                  # captured once, then replayed
        b.lib.bp_solver_set_params(b.handle, p)  # forces a new capture every call
        b.update(2, DT, 4)
    np.testing.assert_array_equal(a.positions(), b.positions())
    assert a.last_launch_count() > 10
    a.close()
    b.close()


def test_picking_matches_oracle(bp, gpu, oracle):
    scene = fluid_scene(bp, (6, 6, 6), seed=2, grid_dim=16)
    params = bp.make_params(scene)
    g = bp.ParticleSolver(scene, params)
    o = oracle.OracleSolver(scene, params)
    pp = np.array([0.5, 1.5, 0.5], np.float32)
    pv = np.array([1.0, 0.0, 0.0], np.float32)
    g.update(2, DT, 3, picked_original_id=7, picked_position=pp, picked_velocity=pv)
    o.update(2, DT, 3, picked=7, picked_position=pp, picked_velocity=pv)
    h = scene.kernel_radius
    assert np.abs(g.positions() - o.positions()).max() <= 1e-4 * h
    np.testing.assert_allclose(g.velocities()[7], pv)
    g.close()


def test_api_queries_and_copies(bp, gpu):
    abi = bp.abi
    scene = small_mixed_scene(bp, seed=12)
    g = bp.ParticleSolver(scene, bp.make_params(scene))
    g.update(2, DT, 2)
    to_orig = g.field(abi.BP_FIELD_MAP_TO_ORIGINAL)
    to_new = g.field(abi.BP_FIELD_MAP_TO_NEW)
    n = scene.num_particles
    assert sorted(to_orig.tolist()) == list(range(n))
    np.testing.assert_array_equal(to_new[to_orig], np.arange(n))
    for i in (0, 5, n - 1):
        assert g.queryOriginalParticleId(i) == to_orig[i]
        assert g.queryNewParticleId(int(to_orig[i])) == i
    xs = g.positions(abi.BP_ORDER_SORTED)
    xo = g.positions(abi.BP_ORDER_ORIGINAL)
    np.testing.assert_array_equal(xo[to_orig], xs)
    np.testing.assert_array_equal(g.getParticlePosition(3), xs[3])
    np.testing.assert_array_equal(g.getParticlePosition(n + 5), np.zeros(3, np.float32))
    # set_state round trip
    g.set_state(xo + 1.0, np.zeros_like(xo))
    np.testing.assert_allclose(g.positions(), xo + 1.0)
    # render records
    out = gpu.empty((n, 4), dtype=gpu.float32, device="cuda:0")
    g.pack_particle_infos(out.data_ptr())
    gpu.cuda.synchronize()
    rec = out.cpu().numpy()
    np.testing.assert_array_equal(rec[:, :3], g.positions(abi.BP_ORDER_SORTED))
    np.testing.assert_array_equal(rec[:, 3].view(np.int32), scene.phases[to_orig])
    # cell offsets are a prefix table of the sorted keys
    off = g.field(abi.BP_FIELD_CELL_OFFSETS)
    keys = g.field(abi.BP_FIELD_SORTED_CELL_IDS)
    assert (np.diff(keys) >= 0).all()
    idx = np.arange(n)
    assert (off[keys] <= idx).all() and (idx < off[keys + 1]).all()
    assert g.device_errors() == 0
    g.close()


def test_nonfinite_state_sets_device_error(bp, gpu):
    scene = fluid_scene(bp, (4, 4, 4), seed=1, grid_dim=16)
    g = bp.ParticleSolver(scene, bp.make_params(scene))
    x = g.positions()
    x[3] = np.nan
    g.set_state(x)
    g.update(1, DT, 1)
    assert g.device_errors() & bp.abi.BP_DEVERR_NONFINITE
    g.close()


def test_empty_scene_update_is_noop(bp, gpu):
    scene = bp.scenes.Scene()
    scene.grid_dim = 16
    scene.kernel_radius = scene.cell_size = 0.2
    g = bp.ParticleSolver(scene, bp.make_params(scene))
    g.update(2, DT, 4)
    assert g.positions().shape == (0, 3)
    g.close()


def test_million_particles_properties(bp, gpu):
    """Full-size fluid block (1,048,576 particles): size-independent checks."""
    abi = bp.abi
    scene = bp.scenes.pbf_scene(128, 64, 128, spacing=0.1, seed=0, box=(12.9, 16.0, 12.9))
    g = bp.ParticleSolver(scene, bp.make_params(scene))
    g.update(2, DT, 4)
    n = scene.num_particles
    keys = g.field(abi.BP_FIELD_SORTED_CELL_IDS)
    to_orig = g.field(abi.BP_FIELD_MAP_TO_ORIGINAL)
    to_new = g.field(abi.BP_FIELD_MAP_TO_NEW)
    off = g.field(abi.BP_FIELD_CELL_OFFSETS)
    assert (np.diff(keys) >= 0).all()
    np.testing.assert_array_equal(to_new[to_orig], np.arange(n))
    assert off[0] == 0 and off[-1] == n and (np.diff(off) >= 0).all()
    x = g.positions()
    assert np.isfinite(x).all() and g.device_errors() == 0
    assert x[:, 1].min() >= 0.0 - 1e-3
    g.close()
