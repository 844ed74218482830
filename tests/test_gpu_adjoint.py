"""Adjoint of the solver step (bp_solver_backward) on the GPU through the C ABI.

Gradients of a loss of the final state are compared with central finite
differences of the same forward solver (directional derivatives along random
directions, so every component of a gradient vector takes part), on short
rollouts where the dynamics are smooth.  The forward runs in fp32, so a
perturbed rollout rounds differently everywhere and the loss carries about
1e-5 of absolute noise; the steps below are large enough that this noise and
the O(eps^2) truncation both stay under the 0.5 % tolerance (measured: 0.02 %
for positions and velocities, at most 0.4 % for wind and stiffness).
Checkpoint spacing must not change the result, and the solver's state must be
as it was after backward."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0
FD_REL = 5e-3  # |fd - adjoint| <= FD_REL * scale, scale = max(|fd|, |adjoint|, floor)


def cloth_case(bp, n=10):
    abi = bp.abi
    scene = bp.scenes.flag_scene(n=n, seed=3, mass=0.05)  # light, so that the wind moves it
    stages = abi.BP_STAGE_PLANES | abi.BP_STAGE_WIND | abi.BP_STAGE_DISTANCE | abi.BP_STAGE_IMMOVABLE
    params = bp.make_params(scene, mode=abi.BP_MODE_TEXTBOOK, stage_mask=stages, wind_velocity=(4.0, 0.0, 1.0),
                            wind_drag=1.0, wind_lift=0.3)
    return scene, params


def fluid_case(bp, n=6):
    abi = bp.abi
    scene = bp.scenes.pbf_scene(n, n, n, spacing=0.1, seed=5, box=(1.2, 2.0, 1.2), grid_dim=16)
    rng = np.random.default_rng(6)
    scene.velocities = rng.uniform(-0.2, 0.2, (scene.num_particles, 3)).astype(np.float32)
    stages = abi.BP_STAGE_FLUID | abi.BP_STAGE_PLANES | abi.BP_STAGE_XSPH
    return scene, bp.make_params(scene, stage_mask=stages)


def rollout(bp, scene, params, updates, substeps=2, iterations=4):
    s = bp.ParticleSolver(scene, params)
    for _ in range(updates):
        s.update(substeps, DT, iterations)
    x, v = s.positions(), s.velocities()
    s.close()
    return x, v


def loss_weights(n, seed=11):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n, 3)).astype(np.float32), rng.standard_normal((n, 3)).astype(np.float32) * 0.1


def loss(x, v, wx, wv):
    return float(np.sum(x.astype(np.float64) * wx) + np.sum(v.astype(np.float64) * wv))


def adjoint(bp, scene, params, updates, wx, wv, every=2, substeps=2, iterations=4):
    s = bp.ParticleSolver(scene, params)
    s.tape_begin(every)
    for _ in range(updates):
        s.update(substeps, DT, iterations)
    g = s.backward(wx, wv)
    s.close()
    return g


def check_dir(fd, ad, floor):
    scale = max(abs(fd), abs(ad), floor)
    assert abs(fd - ad) <= FD_REL * scale, f"finite difference {fd:.6e} vs adjoint {ad:.6e}"


def test_cloth_gradients_match_finite_differences(bp, gpu):
    import copy

    scene, params = cloth_case(bp)
    updates = 3
    wx, wv = loss_weights(scene.num_particles)
    g = adjoint(bp, scene, params, updates, wx, wv)
    rng = np.random.default_rng(21)

    def L(sc, pr):
        return loss(*rollout(bp, sc, pr, updates), wx, wv)

    pairs = []  # (what, eps, finite difference, adjoint)
    # wind velocity (textbook wind is relative to it)
    for eps in (0.2,):
        for k in range(3):
            pp, pm = copy.copy(params), copy.copy(params)
            pp.wind_velocity[k] += eps
            pm.wind_velocity[k] -= eps
            pairs.append((f"wind[{k}]", eps, (L(scene, pp) - L(scene, pm)) / (2 * eps), float(g["wind_velocity"][k])))
    # stiffness of every distance constraint, along one random direction
    d = rng.standard_normal(scene.num_distance_constraints).astype(np.float32)
    d /= np.linalg.norm(d)
    for eps in (4e-2,):
        sp, sm = copy.deepcopy(scene), copy.deepcopy(scene)
        sp.distance_params[:, 1] += eps * d
        sm.distance_params[:, 1] -= eps * d
        pairs.append(("stiffness", eps, (L(sp, params) - L(sm, params)) / (2 * eps),
                      float(g["distance_stiffness"] @ d)))
    # initial velocities and positions
    for key, e0 in (("velocities", 4e-2), ("positions", 4e-3)):
        d = rng.standard_normal((scene.num_particles, 3)).astype(np.float32)
        d /= np.linalg.norm(d)
        for eps in (e0,):
            sp, sm = copy.deepcopy(scene), copy.deepcopy(scene)
            setattr(sp, key, (getattr(scene, key) + eps * d).astype(np.float32))
            setattr(sm, key, (getattr(scene, key) - eps * d).astype(np.float32))
            pairs.append((key, eps, (L(sp, params) - L(sm, params)) / (2 * eps), float(np.sum(g[key] * d))))
    report = "; ".join(f"{w}@{e:g} {fd:.5e}/{ad:.5e}" for w, e, fd, ad in pairs)
    print(report)
    floor = 1e-2 * max(abs(a) for _, _, _, a in pairs)
    bad = [f"{w}@{e:g}: fd {fd:.6e} adjoint {ad:.6e}" for w, e, fd, ad in pairs
           if abs(fd - ad) > FD_REL * max(abs(fd), abs(ad), floor)]
    assert not bad, "; ".join(bad) + " | all: " + report


def test_fluid_gradients_match_finite_differences(bp, gpu):
    """Reference-mode position-based fluid with planes and XSPH: gradient of the
    final centre of mass with respect to the initial velocity field."""
    import copy

    scene, params = fluid_case(bp)
    n = scene.num_particles
    updates = 2
    wx = np.zeros((n, 3), np.float32)
    wx[:, 0] = 1.0 / n  # loss: x of the centre of mass
    wx[:, 1] = 0.5 / n
    wv = np.zeros((n, 3), np.float32)
    g = adjoint(bp, scene, params, updates, wx, wv, iterations=3)
    rng = np.random.default_rng(31)
    for trial in range(2):
        d = rng.standard_normal((n, 3)).astype(np.float32)
        d /= np.linalg.norm(d)
        eps = 2e-2
        sp, sm = copy.deepcopy(scene), copy.deepcopy(scene)
        sp.velocities = (scene.velocities + eps * d).astype(np.float32)
        sm.velocities = (scene.velocities - eps * d).astype(np.float32)
        fd = (loss(*rollout(bp, sp, params, updates, iterations=3), wx, wv) -
              loss(*rollout(bp, sm, params, updates, iterations=3), wx, wv)) / (2 * eps)
        check_dir(fd, float(np.sum(g["velocities"] * d)), 1e-4)


def test_fluid_gradients_on_an_aliased_table(bp, gpu):
    """A 1 m fluid block on a 4^3 table (0.8 m period): the forward walks
    take the alias classes; the adjoint's walks take whole table cells and
    give the gradients of a run without classes, bit for bit."""
    abi = bp.abi
    scene = bp.scenes.pbf_scene(10, 6, 10, spacing=0.1, seed=7, box=(1.4, 2.0, 1.4), grid_dim=4)
    rng = np.random.default_rng(9)
    scene.velocities = rng.uniform(-0.2, 0.2, (scene.num_particles, 3)).astype(np.float32)
    stages = abi.BP_STAGE_FLUID | abi.BP_STAGE_PLANES | abi.BP_STAGE_XSPH
    wx, wv = loss_weights(scene.num_particles, seed=3)
    grads = []
    for w in (abi.BP_WALK_NO_STAGING, abi.BP_WALK_NO_STAGING | abi.BP_WALK_NO_ALIAS_CLASSES):
        params = bp.make_params(scene, stage_mask=stages, walk_options=w)
        s = bp.ParticleSolver(scene, params)
        walks = s.walk_stats(2, DT, 3)  # a real update, then the recorded ones
        assert (walks["alias_classes"] > 0) == (not w & abi.BP_WALK_NO_ALIAS_CLASSES), walks
        s.tape_begin(2)
        for _ in range(2):
            s.update(2, DT, 3)
        grads.append(s.backward(wx, wv))
        s.close()
    for k in grads[0]:
        np.testing.assert_array_equal(grads[0][k], grads[1][k], err_msg=k)


def rigid_case(bp):
    abi = bp.abi
    sc = bp.scenes
    s = sc.Scene(name="rigid_air")
    s.particle_radius, s.kernel_radius, s.cell_size, s.grid_dim, s.rest_density = 0.05, 0.2, 0.2, 32, 1000.0
    s.add_plane((0.0, -20.0, 0.0), (0.0, 1.0, 0.0))
    s.add_rigid_box((3, 3, 3), (0.0, 2.0, 0.0), (0.1, 0.1, 0.1), 1.0)
    s.add_rigid_box((4, 2, 3), (1.0, 2.5, 0.3), (0.1, 0.1, 0.1), 1.0)
    rng = np.random.default_rng(8)
    s.velocities = rng.uniform(-0.5, 0.5, (s.num_particles, 3)).astype(np.float32)  # spins the boxes
    return s, bp.make_params(s, stage_mask=abi.BP_STAGE_PLANES | abi.BP_STAGE_SHAPE_MATCHING)


def test_rigid_gradients_match_finite_differences(bp, gpu):
    """Shape matching, its rotation differentiated at the fixed point of the
    extraction: initial velocities and positions of two spinning boxes."""
    import copy

    scene, params = rigid_case(bp)
    updates = 3
    wx, wv = loss_weights(scene.num_particles, seed=12)
    g = adjoint(bp, scene, params, updates, wx, wv)
    rng = np.random.default_rng(41)
    pairs = []
    # The extraction stops once its rotation step is below 3e-5 rad, so the
    # forward map has jumps of that size: small steps (and deforming position
    # directions) put those jumps into the quotient.  Velocities along a random
    # direction with a 0.16 step, positions along rigid per-body translations.
    body = np.zeros(scene.num_particles, np.int64)
    for b, (r0, r1) in enumerate(scene.rigid_ranges):
        body[r0:r1] = b
    for key, eps0 in (("velocities", 0.16), ("positions", 0.016)):
        if key == "velocities":
            d = rng.standard_normal((scene.num_particles, 3)).astype(np.float32)
        else:
            d = rng.standard_normal((len(scene.rigid_ranges), 3)).astype(np.float32)[body]
        d /= np.linalg.norm(d)
        for eps in (eps0,):
            sp, sm = copy.deepcopy(scene), copy.deepcopy(scene)
            setattr(sp, key, (getattr(scene, key) + eps * d).astype(np.float32))
            setattr(sm, key, (getattr(scene, key) - eps * d).astype(np.float32))
            fd = (loss(*rollout(bp, sp, params, updates), wx, wv) -
                  loss(*rollout(bp, sm, params, updates), wx, wv)) / (2 * eps)
            pairs.append((f"{key}@{eps:g}", fd, float(np.sum(g[key] * d))))
    report = "; ".join(f"{w} {fd:.5e}/{ad:.5e}" for w, fd, ad in pairs)
    print(report)
    floor = 1e-2 * max(abs(a) for _, _, a in pairs)
    bad = [w for w, fd, ad in pairs if abs(fd - ad) > FD_REL * max(abs(fd), abs(ad), floor)]
    assert not bad, report


def test_checkpoint_spacing_does_not_change_gradients(bp, gpu):
    scene, params = cloth_case(bp, n=8)
    wx, wv = loss_weights(scene.num_particles, seed=5)
    ref = adjoint(bp, scene, params, 4, wx, wv, every=1)
    for every in (3, 100):
        g = adjoint(bp, scene, params, 4, wx, wv, every=every)
        for k in ref:
            np.testing.assert_array_equal(ref[k], g[k], err_msg=f"{k}, checkpoint every {every}")


def test_backward_restores_the_state(bp, gpu):
    scene, params = cloth_case(bp, n=8)
    wx, wv = loss_weights(scene.num_particles)
    a = bp.ParticleSolver(scene, params)
    b = bp.ParticleSolver(scene, params)
    a.tape_begin(2)
    for s in (a, b):
        for _ in range(3):
            s.update(2, DT, 4)
    a.backward(wx, wv)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.velocities(), b.velocities())
    for s in (a, b):
        s.update(2, DT, 4)
    np.testing.assert_array_equal(a.positions(), b.positions())
    a.tape_end()
    a.close()
    b.close()


def test_backward_without_a_recording_is_refused(bp, gpu):
    scene, _ = fluid_case(bp, n=4)
    t = bp.ParticleSolver(scene, bp.make_params(scene))
    with pytest.raises(bp.BrassPanError):
        t.backward(np.ones((scene.num_particles, 3), np.float32))  # nothing recorded
    t.close()


# ---- against central finite differences of the FP64 host oracle -------------
#
# The configuration's check: gradients of the GPU adjoint (fp32 forward and
# adjoint) against central differences with step 1e-3 of the FP64 oracle's
# forward (the same step in double; state, wind and stiffness perturbed in
# double), within 1e-3 relative.  A reduced differentiable-rollout
# configuration: a 16 x 16 flag pinned along one edge under wind (4, 0, 0)
# m/s for 20 frames of 2 substeps x 4 iterations, loss = mean squared
# distance of the final positions to a seeded target pose, checkpoints every
# 10 substeps; and an 8^3 PBF block (reference mode, planes, XSPH) for 5
# frames, loss = its final centre of mass.
#
# The flag's loss is curved enough that the step-1e-3 central difference
# itself is off by 2-3e-4 relative at 20-30 frames (measured against step
# 1e-4), so the differences are Richardson-extrapolated from steps 1e-3 and
# 5e-4 ((4 D(h/2) - D(h)) / 3, error O(h^4)).  The adjoint linearises the
# fp32 trajectory, the differences the FP64 one; measured on the flag, the
# initial-velocity direction agrees to 1.5e-5 at 5 frames, 3e-4 at 10-20 and
# 1.04e-3 at 30 frames (wind and stiffness: 1e-4 to 2e-4 throughout).

FD64_STEP = 1e-3
FD64_REL = 1e-3


def central64(L, plus, minus, h=FD64_STEP):
    """Richardson-extrapolated central difference: plus(s) / minus(s) give
    the perturbed arguments of L at step s."""
    d = [(L(**plus(s)) - L(**minus(s))) / (2 * s) for s in (h, h / 2)]
    return (4 * d[1] - d[0]) / 3


def rollout64(oracle, scene, params, updates, x0=None, v0=None, wind=None, dparams=None, iterations=4):
    """Final (positions, velocities) of the FP64 oracle, float64, original order."""
    import os

    o = oracle.OracleSolver(scene, params, threads=os.cpu_count() or 4, precision=64)
    if x0 is not None or v0 is not None:  # a new solver's arrangement is the original order
        o.set_state(x0, v0)
    if wind is not None:
        o.set_wind(wind)
    if dparams is not None:
        o.set_distance_params(dparams)
    for _ in range(updates):
        o.update(2, DT, iterations)
    return o.positions(), o.velocities()


def flag64_case(bp):
    abi = bp.abi
    scene = bp.scenes.flag_scene(n=16, seed=4)
    stages = abi.BP_STAGE_PLANES | abi.BP_STAGE_WIND | abi.BP_STAGE_DISTANCE | abi.BP_STAGE_IMMOVABLE
    params = bp.make_params(scene, mode=abi.BP_MODE_TEXTBOOK, stage_mask=stages, wind_velocity=(4.0, 0.0, 0.0),
                            wind_drag=1.0, wind_lift=0.3, mass_scaling_k=0.0)
    rng = np.random.default_rng(40)
    target = scene.positions.astype(np.float64) + rng.normal(0.0, 0.05, (scene.num_particles, 3))
    return scene, params, target


def test_flag_gradients_match_fp64_finite_differences(bp, gpu, oracle):
    scene, params, target = flag64_case(bp)
    n, frames = scene.num_particles, 20
    s = bp.ParticleSolver(scene, params)
    s.tape_begin(10)
    for _ in range(frames):
        s.update(2, DT, 4)
    x = s.positions().astype(np.float64)
    g = s.backward(((2.0 / n) * (x - target)).astype(np.float32))
    s.close()

    def L(**kw):
        xf, _ = rollout64(oracle, scene, params, frames, **kw)
        return float(np.sum((xf - target) ** 2) / n)

    x0 = scene.positions.astype(np.float64)
    v0 = np.zeros((n, 3)) if scene.velocities is None else scene.velocities.astype(np.float64)
    wind = np.array(params.wind_velocity[:], np.float64)
    dp = scene.distance_params.astype(np.float64)
    rng = np.random.default_rng(42)
    pairs = []
    for k in range(3):
        e = np.zeros(3)
        e[k] = 1.0
        pairs.append((f"wind[{k}]", central64(L, lambda s: {"wind": wind + s * e}, lambda s: {"wind": wind - s * e}),
                      float(g["wind_velocity"][k])))
    d = rng.standard_normal(len(dp))
    d /= np.linalg.norm(d)
    ds = np.zeros_like(dp)
    ds[:, 1] = d
    pairs.append(("stiffness", central64(L, lambda s: {"dparams": dp + s * ds}, lambda s: {"dparams": dp - s * ds}),
                  float(g["distance_stiffness"].astype(np.float64) @ d)))
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d)
    pairs.append(("velocities", central64(L, lambda s: {"x0": x0, "v0": v0 + s * d},
                                          lambda s: {"x0": x0, "v0": v0 - s * d}),
                  float(np.sum(g["velocities"].astype(np.float64) * d))))
    report = "; ".join(f"{w} fd64 {fd:.6e} adjoint {ad:.6e}" for w, fd, ad in pairs)
    print(report)
    floor = 1e-2 * max(abs(a) for _, _, a in pairs)
    bad = [w for w, fd, ad in pairs if abs(fd - ad) > FD64_REL * max(abs(fd), abs(ad), floor)]
    assert not bad, report


def test_pbf_block_gradient_matches_fp64_finite_differences(bp, gpu, oracle):
    abi = bp.abi
    scene = bp.scenes.pbf_scene(8, 8, 8, spacing=0.1, seed=4, box=(1.6, 2.0, 1.6), grid_dim=16)
    params = bp.make_params(scene, stage_mask=abi.BP_STAGE_FLUID | abi.BP_STAGE_PLANES | abi.BP_STAGE_XSPH)
    n, frames = scene.num_particles, 5
    s = bp.ParticleSolver(scene, params)
    s.tape_begin(10)
    for _ in range(frames):
        s.update(2, DT, 4)
    gx = np.full((n, 3), 1.0 / n, np.float32)  # loss: sum of the centre of mass's coordinates
    g = s.backward(gx)
    s.close()

    def L(v0):
        xf, _ = rollout64(oracle, scene, params, frames, x0=scene.positions.astype(np.float64), v0=v0)
        return float(xf.sum() / n)

    v0 = np.zeros((n, 3)) if scene.velocities is None else scene.velocities.astype(np.float64)
    rng = np.random.default_rng(43)
    pairs = []
    for trial in range(2):
        d = rng.standard_normal((n, 3))
        d /= np.linalg.norm(d)
        pairs.append((f"velocities#{trial}", central64(L, lambda s: {"v0": v0 + s * d}, lambda s: {"v0": v0 - s * d}),
                      float(np.sum(g["velocities"].astype(np.float64) * d))))
    report = "; ".join(f"{w} fd64 {fd:.6e} adjoint {ad:.6e}" for w, fd, ad in pairs)
    print(report)
    bad = [w for w, fd, ad in pairs if abs(fd - ad) > FD64_REL * max(abs(fd), abs(ad))]
    assert not bad, report


# ---- the remaining stages against FP64 finite differences ---------------------
#
# Particle contacts with friction, vorticity confinement with Akinci tension
# (reference mode, through the density of the last lambda pass), and dihedral
# bending: each on a small scene over a few substeps, loss = random weights on
# the final positions and velocities, directional derivatives along random
# unit directions of the initial velocities (step 1e-3) and positions.
#
# The step map is only piecewise smooth in the positions: reference-mode
# density sums over sorted j >= i, so it jumps where a particle crosses a cell
# boundary, vorticity confinement switches on where |eta|^2 passes 1e-3, and
# contact friction switches between its static and kinetic forms.  Along a
# position direction, steps of 1e-3 to 1e-5 straddle such jumps in these
# scenes (measured: the quotient changes sign between them), so positions are
# differenced at step 1e-6 (the same quotient as at 1e-7 to 7 digits; the
# FP64 forward resolves it to about 1e-9); the scenes start away from cell
# boundaries.


def fd64_state_pairs(oracle, scene, params, frames, wx, wv, g, seed, x_step=1e-6):
    def L(x0, v0):
        xf, vf = rollout64(oracle, scene, params, frames, x0=x0, v0=v0)
        return float(np.sum(xf * wx) + np.sum(vf * wv))

    n = scene.num_particles
    x0 = scene.positions.astype(np.float64)
    v0 = np.zeros((n, 3)) if scene.velocities is None else scene.velocities.astype(np.float64)
    rng = np.random.default_rng(seed)
    pairs = []
    for key in ("velocities", "positions"):
        d = rng.standard_normal((n, 3))
        d /= np.linalg.norm(d)
        if key == "velocities":
            fd = central64(lambda **kw: L(**kw), lambda s: {"x0": x0, "v0": v0 + s * d},
                           lambda s: {"x0": x0, "v0": v0 - s * d})
        else:
            fd = central64(lambda **kw: L(**kw), lambda s: {"x0": x0 + s * d, "v0": v0},
                           lambda s: {"x0": x0 - s * d, "v0": v0}, h=x_step)
        pairs.append((key, fd, float(np.sum(g[key].astype(np.float64) * d))))
    return pairs


def assert_fd64(pairs):
    report = "; ".join(f"{w} fd64 {fd:.6e} adjoint {ad:.6e}" for w, fd, ad in pairs)
    print(report)
    floor = 1e-2 * max(abs(a) for _, _, a in pairs)
    bad = [w for w, fd, ad in pairs if abs(fd - ad) > FD64_REL * max(abs(fd), abs(ad), floor)]
    assert not bad, report


def gpu_gradients(bp, scene, params, frames, wx, wv, every=2):
    s = bp.ParticleSolver(scene, params)
    s.tape_begin(every)
    for _ in range(frames):
        s.update(2, DT, 4)
    g = s.backward(wx.astype(np.float32), wv.astype(np.float32))
    s.close()
    return g


def grains_case(bp, fluid=False):
    """A block of grains (single-particle solids) packed closer than two radii,
    so that every grain starts in contact; optionally over a small fluid pool."""
    abi = bp.abi
    sc = bp.scenes
    rng = np.random.default_rng(9)
    s = sc.Scene(name="grains")
    s.particle_radius, s.kernel_radius, s.cell_size, s.grid_dim, s.rest_density = 0.05, 0.2, 0.2, 16, 1000.0
    sc.box_planes(s, (0, 0, 0), (1.6, 3.0, 1.6))
    stages = abi.BP_STAGE_PLANES | abi.BP_STAGE_PARTICLE_COLLISION
    if fluid:
        s.add_fluid_block((8, 3, 8), (0.35, 0.05, 0.35), (0.1, 0.1, 0.1), 1.0, jitter=0.001, rng=rng)
        stages |= abi.BP_STAGE_FLUID
    s.add_granulars_block((4, 4, 4), (0.65, 0.45 if fluid else 0.35, 0.65), (0.09, 0.09, 0.09), 1.0)
    s.velocities = rng.uniform(-0.3, 0.3, (s.num_particles, 3)).astype(np.float32)
    return s, bp.make_params(s, stage_mask=stages)


@pytest.mark.parametrize("fluid", [False, True], ids=["grains", "grains_on_fluid"])
def test_contact_gradients_match_fp64_finite_differences(bp, gpu, oracle, fluid):
    scene, params = grains_case(bp, fluid)
    frames = 2
    wx, wv = loss_weights(scene.num_particles, seed=21)
    g = gpu_gradients(bp, scene, params, frames, wx, wv)
    assert_fd64(fd64_state_pairs(oracle, scene, params, frames, wx, wv, g, seed=22))


def test_vorticity_and_akinci_gradients_match_fp64_finite_differences(bp, gpu, oracle):
    abi = bp.abi
    scene = bp.scenes.pbf_scene(6, 6, 6, spacing=0.1, seed=7, box=(1.2, 2.0, 1.2), grid_dim=16)
    scene.positions = (scene.positions + np.float32(0.05)).astype(np.float32)  # off the cell boundaries
    rng = np.random.default_rng(8)
    scene.velocities = rng.uniform(-0.5, 0.5, (scene.num_particles, 3)).astype(np.float32)
    stages = (abi.BP_STAGE_FLUID | abi.BP_STAGE_PLANES | abi.BP_STAGE_VORTICITY | abi.BP_STAGE_AKINCI |
              abi.BP_STAGE_XSPH)
    params = bp.make_params(scene, stage_mask=stages)
    frames = 2
    wx, wv = loss_weights(scene.num_particles, seed=23)
    g = gpu_gradients(bp, scene, params, frames, wx, wv)
    assert_fd64(fd64_state_pairs(oracle, scene, params, frames, wx, wv, g, seed=24))


def twisted_cloth(bp):
    """The pinned cloth of the bending tests, twisted (height 0.8 (x - cx)(z - cz)),
    so that every hinge starts about 0.1 rad from flat and stays above 0.03
    rad over the rollout.  Near flat the reference's bending term cannot be
    differentiated in fp32: its dihedral cosine d rounds to -1 within 3.5e-4
    rad of flat, where sqrt(1 - d^2) is then a few rounding steps of 1 + d,
    so the fp32 forward's slope there is rounding noise (measured on the
    initially flat cloth: 2-100 % from the FP64 differences, while without
    bending the same rollout agrees to 4e-5)."""
    from conftest import cloth_bending_scene

    scene = cloth_bending_scene(bp, seed=3, n=8)
    x = scene.positions.astype(np.float64)
    c = x[:, [0, 2]].mean(axis=0)
    x[:, 1] += 0.8 * (x[:, 0] - c[0]) * (x[:, 2] - c[1])
    scene.positions = x.astype(np.float32)
    return scene


def test_bending_gradients_match_fp64_finite_differences(bp, gpu, oracle):
    abi = bp.abi
    scene = twisted_cloth(bp)
    stages = abi.BP_STAGE_PLANES | abi.BP_STAGE_DISTANCE | abi.BP_STAGE_BENDING | abi.BP_STAGE_IMMOVABLE
    params = bp.make_params(scene, stage_mask=stages, bending_stiffness=0.2)
    frames = 2
    wx, wv = loss_weights(scene.num_particles, seed=25)
    g = gpu_gradients(bp, scene, params, frames, wx, wv)
    assert_fd64(fd64_state_pairs(oracle, scene, params, frames, wx, wv, g, seed=26, x_step=FD64_STEP))  # smooth


def test_textbook_fluid_gradients_match_fp64_finite_differences(bp, gpu, oracle):
    """Textbook mode: density over all neighbours, the exact lambda denominator
    (its gradient norms differentiated through the spiky Hessian), s_corr, and
    XSPH weighted by m_j / rho_j, whose density gradient joins the last lambda
    pass's; with vorticity and Akinci tension."""
    abi = bp.abi
    scene = bp.scenes.pbf_scene(6, 6, 6, spacing=0.1, seed=11, box=(1.2, 2.0, 1.2), grid_dim=16)
    scene.positions = (scene.positions + np.float32(0.05)).astype(np.float32)  # off the cell boundaries
    rng = np.random.default_rng(12)
    scene.velocities = rng.uniform(-0.5, 0.5, (scene.num_particles, 3)).astype(np.float32)
    stages = (abi.BP_STAGE_FLUID | abi.BP_STAGE_PLANES | abi.BP_STAGE_VORTICITY | abi.BP_STAGE_AKINCI |
              abi.BP_STAGE_XSPH)
    params = bp.make_params(scene, mode=abi.BP_MODE_TEXTBOOK, stage_mask=stages)
    frames = 2
    wx, wv = loss_weights(scene.num_particles, seed=27)
    g = gpu_gradients(bp, scene, params, frames, wx, wv)
    assert_fd64(fd64_state_pairs(oracle, scene, params, frames, wx, wv, g, seed=28))


def test_picking_gradients_match_fp64_finite_differences(bp, gpu, oracle):
    """Picking: the picked particle is set to its target at the start of every
    substep and of every iteration, and given the picked velocity after the
    update, so nothing before those reaches the loss through it; the other
    particles' gradients flow through its constraints."""
    import os

    scene, params = cloth_case(bp)
    n, frames, pick = scene.num_particles, 3, 44
    target = (scene.positions[pick] + np.array([0.05, 0.1, -0.03])).astype(np.float32)
    pvel = np.array([0.5, 0.0, 0.2], np.float32)
    wx, wv = loss_weights(n, seed=29)
    s = bp.ParticleSolver(scene, params)
    s.tape_begin(2)
    for _ in range(frames):
        s.update(2, DT, 4, picked_original_id=pick, picked_position=target, picked_velocity=pvel)
    g = s.backward(wx, wv)
    s.close()
    assert np.all(g["positions"][pick] == 0) and np.all(g["velocities"][pick] == 0)

    def L(x0, v0):
        o = oracle.OracleSolver(scene, params, threads=os.cpu_count() or 4, precision=64)
        o.set_state(x0, v0)
        for _ in range(frames):
            o.update(2, DT, 4, picked=pick, picked_position=target, picked_velocity=pvel)
        return float(np.sum(o.positions() * wx) + np.sum(o.velocities() * wv))

    x0 = scene.positions.astype(np.float64)
    v0 = np.zeros((n, 3)) if scene.velocities is None else scene.velocities.astype(np.float64)
    rng = np.random.default_rng(30)
    pairs = []
    for key in ("velocities", "positions"):
        d = rng.standard_normal((n, 3))
        d /= np.linalg.norm(d)
        if key == "velocities":
            fd = central64(lambda **kw: L(**kw), lambda h: {"x0": x0, "v0": v0 + h * d},
                           lambda h: {"x0": x0, "v0": v0 - h * d})
        else:
            fd = central64(lambda **kw: L(**kw), lambda h: {"x0": x0 + h * d, "v0": v0},
                           lambda h: {"x0": x0 - h * d, "v0": v0})
        pairs.append((key, fd, float(np.sum(g[key].astype(np.float64) * d))))
    assert_fd64(pairs)
