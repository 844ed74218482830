"""Throughput benchmark: particle-substeps/s of the solver step on one GB300.

A step is one call of update(2 substeps, dt = 1/60 s, 4 iterations) (one
frame) on the mixed-phase scene of the benchmark configuration (1,048,576 PBF
fluid particles, a 256x256 cloth under wind, 64 rigid 8^3 cubes; 1,146,880
particles), reference-mode parameters.  W warm-up frames, the walk autotuner,
then K timed frames (CUDA events, L2 flushed before each).  Its "e2e" object
replays the same frames through the C ABI, each frame's state uploaded from
pinned host memory and its positions and velocities read back.  Prints one
JSON line, which also carries (each can be switched off):
  reference_cuda  the reference's own CUDA step (its kernel headers built for
                  sm_103a, oracle/ref_cuda.cu) on the same GPU and frames;
  workloads       the other configurations and regimes (32k dam break, the
                  shape-matching stress test, the 1M PBF block, the mixed
                  scene 200 frames in, the mixed scene's textbook parameters);
  batched         256 PBF dam breaks of 4096..262144 particles in one solver
                  against looping one solver per scene;
  adjoint         forward + backward() of differentiable rollouts against the
                  forward alone, with FP64 finite-difference gradient checks;
  cpu_baseline    the reference's kernels compiled for the host, all cores.
`--impl reference` times the reference's step on the host cores (the
reference arm): same workload, warm-up and frames, no product code loaded.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload mixed|fluid|small|batch|rigid] [--no-batch] [--no-adjoint]
                  [--no-reference-cuda] [--no-samples] [--no-gradient-check]

Multi-GPU (torchrun, one rank per GPU): the scene does not shard, so every
rank advances its own replica ("replicas only"); value = all ranks' particle
substeps / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

DT = 1.0 / 60.0
SUBSTEPS = 2
ITERATIONS = 4

# Algorithmic bytes per particle per launch (each per-particle input read
# once, each output written once; neighbour re-reads are cache traffic).
KERNEL_BYTES = {
    "launch_lambda": 16 + 4 + 4 + 4,            # P, mass -> lambda, rho
    "launch_deltap": 16 + 4 + 4 + 16 + 16,      # P, lambda, mass, Xs (planes) -> P'
    "launch_post_a": 16 + 16 + 4 + 16 + 16,     # P, V, rho -> omega, normal
    "launch_post_b": 16 + 16 + 16 + 16 + 16,    # P, V, Om, Nm -> V'
    "launch_post_c": 16 + 16 + 16,              # P, V -> V'
    "launch_particle_collision": 16 + 16 + 4 + 16,
    "launch_reorder": 4 + 16 + 16 + 4 + 16 * 3 + 4 + 4 + 4 + 4,
    "launch_hash_state": 16 + 16 + 4,
}


def load_peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def build_scene(scenes, workload: str, seed: int = 0):
    """The workload's scene from the builders module `scenes`."""
    if workload == "mixed":
        return scenes.mixed_phase_1m(seed=seed)
    if workload == "fluid":
        return scenes.pbf_scene(128, 64, 128, spacing=0.1, seed=seed, box=(12.9, 16.0, 12.9))
    if workload == "small":
        return scenes.pbf_scene(32, 32, 32, spacing=0.1, seed=seed, box=(4.0, 4.0, 4.0))
    if workload == "rigid":
        return scenes.rigid_body_pile(seed=seed)
    if workload == "batch":  # CPU-side sample of the ensemble: its largest member
        return max(scenes.dam_break_ensemble(seed=seed), key=lambda sc: sc.num_particles)
    raise SystemExit(f"unknown workload {workload}")


def workload_name(workload, n):
    return {"mixed": "mixed-phase: 128x64x128 PBF fluid + 256^2 cloth (wind) + 64 rigid 8^3 cubes",
            "fluid": "PBF dam break 128x64x128", "small": "PBF dam break 32^3",
            "batch": "batched ensemble: 256 PBF dam breaks, log-uniform 4096..262144 particles",
            "rigid": "shape-matching stress: 4096 rigid bodies of 27..1000 particles with contacts"}[workload] + f", N={n}"


def timed_steps(torch, stream, flush, steps, fn):
    """CUDA-event time (ms) of `steps` calls of fn on `stream`, L2 flushed before each."""
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        flush.fill_(k & 0xFF)
        starts[k].record(stream)
        fn()
        ends[k].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in zip(starts, ends))


def run_adjoint(bp, torch, stream, frames=120, every=10, check_gradients=True):
    """Differentiable rollouts: a 128x128 cloth flag pinned along one edge
    under wind (4, 0, 0) m/s (loss: squared distance of the final positions to
    a seeded target) and a 64x32x32 = 65,536-particle PBF block (loss: final
    centre of mass), each for `frames` updates of 2 substeps x 4 iterations,
    checkpoints every `every` substeps.  Times one forward rollout and one
    forward rollout recorded on a tape plus backward().  With check_gradients,
    each case's gradient is compared with FP64 finite differences (fd64_check)."""
    abi = bp.abi
    out = {}
    cloth = bp.scenes.flag_scene(n=128, seed=4)
    cloth_stages = abi.BP_STAGE_PLANES | abi.BP_STAGE_WIND | abi.BP_STAGE_DISTANCE | abi.BP_STAGE_IMMOVABLE
    # no mass scaling: exp(2 y) over a 13 m tall flag would span 11 orders of magnitude
    cloth_params = bp.make_params(cloth, mode=abi.BP_MODE_TEXTBOOK, stage_mask=cloth_stages,
                                  wind_velocity=(4.0, 0.0, 0.0), wind_drag=1.0, wind_lift=0.3, mass_scaling_k=0.0)
    fluid = bp.scenes.pbf_scene(64, 32, 32, spacing=0.1, seed=4, box=(9.6, 8.0, 4.8), grid_dim=64)
    fluid_params = bp.make_params(fluid, stage_mask=abi.BP_STAGE_FLUID | abi.BP_STAGE_PLANES | abi.BP_STAGE_XSPH)
    rng = np.random.default_rng(4)
    for name, scene, params in (("cloth_flag_128x128", cloth, cloth_params), ("pbf_block_65536", fluid, fluid_params)):
        n = scene.num_particles
        if name.startswith("cloth"):
            target = scene.positions + rng.normal(0.0, 0.05, (n, 3)).astype(np.float32)
        s = bp.ParticleSolver(scene, params, stream=stream.cuda_stream)
        x0, v0 = s.positions(), s.velocities()
        with torch.cuda.stream(stream):
            s.update(SUBSTEPS, DT, ITERATIONS)  # graph capture outside the timed region
            s.set_state(x0, v0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(frames):
                s.update(SUBSTEPS, DT, ITERATIONS)
            x = s.positions()
            fwd = time.perf_counter() - t0
            s.set_state(x0, v0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.tape_begin(every)
            for _ in range(frames):
                s.update(SUBSTEPS, DT, ITERATIONS)
            x = s.positions()
            if name.startswith("cloth"):
                gx = (2.0 / n) * (x - target)
            else:
                gx = np.zeros((n, 3), np.float32)
                gx[:] = 1.0 / n
            g = s.backward(gx)
            both = time.perf_counter() - t0
            s.tape_end()
        s.close()
        out[name] = {"particles": n, "substeps": frames * SUBSTEPS, "checkpoint_every": every,
                     "forward_ms": fwd * 1e3, "forward_adjoint_ms": both * 1e3, "ratio": both / fwd,
                     "grad_finite": bool(np.isfinite(g["velocities"]).all())}
        if check_gradients:
            # horizons: a short one, where the rollout's derivative is what a
            # finite difference measures, and the configuration's own (cloth)
            # or as long as the FP64 fluid rollouts allow (a quarter second
            # per frame at this size)
            horizons = (20, frames) if name.startswith("cloth") else (2, 10)
            out[name]["gradient_check"] = {
                f"frames_{f}": fd64_check(bp, stream, every, scene, params, f,
                                          target=target if name.startswith("cloth") else None)
                for f in horizons}
    return out


def fd64_check(bp, stream, every, scene, params, frames, target=None, h=1e-3):
    """Directional derivatives of the GPU adjoint over a `frames`-update tape
    against central differences (step h) of the FP64 host oracle's forward,
    along the wind's three axes, one random direction in the per-edge
    stiffness and one in the initial velocities (cloth; loss: mean squared
    distance to `target`), or one random initial-velocity direction (fluid;
    loss: sum of the centre of mass's coordinates).  Each difference is taken
    at steps h and h/2 and Richardson-extrapolated; the plain step-h
    difference is reported beside it, and a plain difference at step 1e-6:
    the fluid's step map jumps where a particle crosses a cell boundary
    (reference-mode density over sorted j >= i), and a long rollout's
    step-h differences straddle such jumps, which the small step mostly
    does not."""
    import oracle

    n = scene.num_particles
    threads = os.cpu_count() or 4
    s = bp.ParticleSolver(scene, params, stream=stream.cuda_stream)
    s.tape_begin(every)
    for _ in range(frames):
        s.update(SUBSTEPS, DT, ITERATIONS)
    if target is not None:
        grads = s.backward(((2.0 / n) * (s.positions().astype(np.float64) - target)).astype(np.float32))
    else:
        grads = s.backward(np.full((n, 3), 1.0 / n, np.float32))
    s.close()

    def loss(**kw):
        o = oracle.OracleSolver(scene, params, threads=threads, precision=64)
        if "v0" in kw:
            o.set_state(scene.positions.astype(np.float64), kw["v0"])
        if "wind" in kw:
            o.set_wind(kw["wind"])
        if "dparams" in kw:
            o.set_distance_params(kw["dparams"])
        for _ in range(frames):
            o.update(SUBSTEPS, DT, ITERATIONS)
        x = o.positions()
        return float(np.sum((x - target) ** 2) / n) if target is not None else float(x.sum() / n)

    small = 1e-6

    def central(arg, base, direction):
        dd = [(loss(**{arg: base + s * direction}) - loss(**{arg: base - s * direction})) / (2 * s)
              for s in (h, h / 2, small)]
        return dd[0], (4 * dd[1] - dd[0]) / 3, dd[2]

    rng = np.random.default_rng(7)
    v0 = (np.zeros((n, 3)) if scene.velocities is None else scene.velocities.astype(np.float64))
    t0 = time.perf_counter()
    rows = []
    if target is not None:
        wind = np.array(params.wind_velocity[:], np.float64)
        for k in range(3):
            rows.append((f"wind[{k}]", *central("wind", wind, np.eye(3)[k]), float(grads["wind_velocity"][k])))
        dp = scene.distance_params.astype(np.float64)
        d = rng.standard_normal(len(dp))
        d /= np.linalg.norm(d)
        ds = np.zeros_like(dp)
        ds[:, 1] = d
        rows.append(("stiffness", *central("dparams", dp, ds),
                     float(grads["distance_stiffness"].astype(np.float64) @ d)))
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d)
    rows.append(("velocities", *central("v0", v0, d), float(np.sum(grads["velocities"].astype(np.float64) * d))))
    rel = {w: abs(fr - ad) / max(abs(fr), 1e-30) for w, _, fr, _, ad in rows}
    rel_plain = {w: abs(fd - ad) / max(abs(fd), 1e-30) for w, fd, _, _, ad in rows}
    rel_small = {w: abs(fs - ad) / max(abs(fs), 1e-30) for w, _, _, fs, ad in rows}
    return {"frames": frames, "fd_step": h, "max_rel_error": max(rel.values()),
            "rel_error": {w: float(r) for w, r in rel.items()},
            "max_rel_error_plain_step": max(rel_plain.values()),
            "max_rel_error_step_1e-6": max(rel_small.values()),
            "fd64": {w: fr for w, _, fr, _, _ in rows}, "fd64_plain_step": {w: fd for w, fd, _, _, _ in rows},
            "fd64_step_1e-6": {w: fs for w, _, _, fs, _ in rows},
            "adjoint": {w: ad for w, _, _, _, ad in rows},
            "oracle": "FP64 host oracle; central differences at steps h and h/2, Richardson-extrapolated "
                      "(the plain step-h and step-1e-6 differences beside it)", "seconds": time.perf_counter() - t0}


# Algorithmic bytes of one PBF particle-substep: 514 + 76 I at I iterations
# (predict + hash 56, sort 16, cell ranges 6, reorder 108, per iteration
# lambda 24 + delta-p with planes 52, velocity + commit 64, vorticity 112,
# Akinci 104, XSPH 48): the whole step's compulsory traffic per particle.
STEP_BYTES_PBF = 514 + 76 * ITERATIONS


def kernel_roofline(torch, solver, n, workload, flush, value, prof_steps=3):
    """Per-kernel device time of `prof_steps` real updates (bp_solver_profile:
    CUDA events after every launch on the solver's stream, L2 flushed before
    each update) and the HBM roofline of the longest-running kernel: its
    algorithmic bytes per launch over its average launch time, against the
    measured copy bandwidth; beside it the step-level fraction of the PBF
    byte model at the measured `value`.  Returns (roofline, stages, ms)."""
    agg: dict[str, list] = {}
    for _ in range(prof_steps):
        flush.fill_(7)
        torch.cuda.synchronize()
        for name, (cnt, tot) in solver.profile(SUBSTEPS, DT, ITERATIONS).items():
            a = agg.setdefault(name, [0, 0.0])
            a[0] += cnt
            a[1] += tot
    top_name, (top_launches, top_ms) = max(agg.items(), key=lambda kv: kv[1][1])
    avg_ms = top_ms / top_launches
    peak, peak_kind = load_peaks()
    bytes_per = KERNEL_BYTES.get(top_name)
    achieved = (bytes_per * n / (avg_ms / 1e3) / 1e9) if bytes_per else None
    step_gbs = STEP_BYTES_PBF * value / 1e9
    roofline = {"bound": "hbm", "kernel": top_name, "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
                "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                "traffic": traffic_for(top_name, n, workload), "bytes_per_particle": bytes_per,
                "avg_launch_ms": avg_ms, "issue": issue_for(top_name, workload),
                "step": {"bytes_per_particle_substep": STEP_BYTES_PBF, "achieved": step_gbs,
                         "frac": step_gbs / peak}}
    stages = {k: round(v[1] / prof_steps, 4) for k, v in sorted(agg.items(), key=lambda kv: -kv[1][1])}
    return roofline, stages, sum(v[1] for v in agg.values()) / prof_steps


def run_sample(bp, torch, stream, flush, local, name, scene, params, frames, warmup, pre_frames=0,
               reference_cuda=False):
    """One more workload, timed like the headline one: `pre_frames` untimed
    updates to reach the regime sampled, `warmup` more, the autotuner, one
    more untimed update, then `frames` timed updates (CUDA events on the
    solver's stream, L2 flushed before each),
    clocks sampled meanwhile; the roofline of its top kernel; and, with
    reference_cuda, the reference's CUDA step timed from the same state."""
    n = scene.num_particles
    solver = bp.ParticleSolver(scene, params, stream=stream.cuda_stream)
    try:
        with torch.cuda.stream(stream):
            for _ in range(pre_frames):
                solver.update(SUBSTEPS, DT, ITERATIONS)
            state = (solver.positions(), solver.velocities()) if (reference_cuda and pre_frames) else None
            for _ in range(warmup):
                solver.update(SUBSTEPS, DT, ITERATIONS)
            opt, _ = solver.autotune(SUBSTEPS, DT, ITERATIONS)  # as the headline workload
            tuned = {"walk_options": opt, "scan_block": int(solver.params.scan_block),
                     "scan_persistent": int(solver.params.scan_persistent)}
            solver.update(SUBSTEPS, DT, ITERATIONS)  # captures the chosen variant's graph
            with ClockSampler(local) as clocks:
                ms = timed_steps(torch, stream, flush, frames, lambda: solver.update(SUBSTEPS, DT, ITERATIONS))
            value = n * SUBSTEPS * frames / (ms / 1e3)
            roofline, stages, _ = kernel_roofline(torch, solver, n, name, flush, value)
            walks = solver.walk_stats(SUBSTEPS, DT, ITERATIONS)
            errors = solver.device_errors()
    finally:
        solver.close()
    out = {"workload": name, "particles": n, "frames_before": pre_frames, "warmup": warmup + 1, "steps": frames,
           "autotune": tuned,
           "value": value, "unit": "particle-substeps/s", "ms_per_step": ms / frames, "roofline": roofline,
           "top_stages_ms_per_step": dict(list(stages.items())[:6]), "neighbor_walks": walks,
           "device_errors": errors, "clocks": clocks.summary()}
    if reference_cuda:
        ref = run_reference_cuda(bp, torch, scene, params, frames, warmup, flush, state=state)
        if ref is not None:
            ref["ours_over_reference"] = value / ref["value"]
            out["reference_cuda"] = ref
    return out


def textbook_mixed_params(bp, scene):
    """The mixed configuration's textbook parameters: PBF with relaxation 600,
    s_corr (n = 4 at 0.2 h; k = 0.001, the configuration's 0.1 diverges at
    rho0 = 1000), XSPH c = 0.01, wind (3, 0, 1) m/s with lift 0.3 and drag
    1.0, Akinci tension 0.5, 10 rotation-extraction iterations."""
    return bp.make_params(scene, mode=bp.abi.BP_MODE_TEXTBOOK, relaxation=600.0, scorr_k=0.001, scorr_n=4,
                          scorr_dq=0.2, xsph_c=0.01, wind_velocity=(3.0, 0.0, 1.0), wind_lift=0.3, wind_drag=1.0,
                          surface_tension=0.5, rotation_iterations=10, mass_scaling_k=0.0)


def run_samples(bp, torch, stream, flush, local, args):
    """The other configurations and regimes, each a sub-object of the line:
    the 32k dam break (its 100 frames, textbook parameters, and reference
    parameters against the reference's CUDA step), the shape-matching stress
    test, the 1M PBF block alone and a 16.8M block 16 times wider (both
    against the reference's CUDA step), the mixed scene 200 frames in (late
    regime: compressed fluid, aliased table) against the reference's CUDA
    step from the same state, and the mixed scene with textbook parameters."""
    sc = bp.scenes
    out = {}
    small = sc.dam_break_32k(seed=0)
    out["small"] = run_sample(bp, torch, stream, flush, local, "small", small,
                              bp.make_params(small, mode=bp.abi.BP_MODE_TEXTBOOK, relaxation=600.0, scorr_k=0.001,
                                             scorr_n=4, scorr_dq=0.2, xsph_c=0.01), frames=100, warmup=3)
    out["small_reference"] = run_sample(bp, torch, stream, flush, local, "small", small,
                                        workload_params(bp, "small", small), frames=100, warmup=3,
                                        reference_cuda=not args.no_reference_cuda)
    rigid = sc.rigid_body_pile(seed=0)
    out["rigid"] = run_sample(bp, torch, stream, flush, local, "rigid", rigid, workload_params(bp, "rigid", rigid),
                              frames=10, warmup=3)
    fluid = build_scene(sc, "fluid", seed=0)
    out["pbf_1m"] = run_sample(bp, torch, stream, flush, local, "fluid", fluid, workload_params(bp, "fluid", fluid),
                               frames=args.steps, warmup=args.warmup, reference_cuda=not args.no_reference_cuda)
    big = sc.pbf_scene(512, 64, 512, spacing=0.1, seed=0, box=(51.4, 16.0, 51.4), grid_dim=256)
    out["pbf_16m"] = run_sample(bp, torch, stream, flush, local, "fluid", big, workload_params(bp, "fluid", big),
                                frames=min(args.steps, 10), warmup=3, reference_cuda=not args.no_reference_cuda)
    del big
    mixed = build_scene(sc, "mixed", seed=0)
    out["late"] = run_sample(bp, torch, stream, flush, local, "mixed", mixed, workload_params(bp, "mixed", mixed),
                             frames=5, warmup=0, pre_frames=200, reference_cuda=not args.no_reference_cuda)
    out["textbook"] = run_sample(bp, torch, stream, flush, local, "mixed", mixed, textbook_mixed_params(bp, mixed),
                                 frames=args.steps, warmup=args.warmup)
    names = {"small": workload_name("small", small.num_particles) + ", textbook parameters, 100 frames",
             "small_reference": workload_name("small", small.num_particles) + ", reference parameters, 100 frames",
             "rigid": workload_name("rigid", rigid.num_particles),
             "pbf_1m": workload_name("fluid", fluid.num_particles) + ", reference parameters",
             "pbf_16m": f"PBF dam break 512x64x512 (the 1M block 16 times wider), 2^24-cell table, "
                        f"N={512 * 64 * 512}, reference parameters, {min(args.steps, 10)} frames after 4 untimed",
             "late": workload_name("mixed", mixed.num_particles) + ", frames 201-205 (after 200 untimed)",
             "textbook": workload_name("mixed", mixed.num_particles) + ", textbook parameters"}
    for k, v in out.items():
        v["workload"] = names[k]
    return out


REFERENCE_MAX_BODY = 64  # NUM_MAX_PARTICLE_PER_RIGID_BODY (kernel/cubrasstower.cuh:22)


def reference_cuda_params(bp, scene, params):
    """The parameters the reference's CUDA step runs a workload with: its
    shape-matching kernel handles at most 64 particles per body, and the
    mixed scene's 512-particle cubes turn its state non-finite in the third
    frame (their centre of mass is the sum of 64 positions over 512, so 64
    particles per cube land inside the fluid).  A scene with larger bodies
    leaves the stage out of the reference's run; ours keeps it."""
    import copy

    p = copy.copy(params)
    sizes = [int(r1 - r0) for r0, r1 in scene.rigid_ranges]
    if sizes and max(sizes) > REFERENCE_MAX_BODY:
        p.stage_mask = int(p.stage_mask) & ~bp.abi.BP_STAGE_SHAPE_MATCHING
    return p


def run_reference_cuda(bp, torch, scene, params, steps, warmup, flush, state=None):
    """The reference's own step on this GPU: its kernel headers compiled by
    nvcc for sm_103a and launched by the replay driver (oracle/ref_cuda.cu) on
    the legacy default stream, same scene, parameters (reference_cuda_params),
    update shape, warm-up and L2 flush as the GPU arm; CUDA events around each
    update.  `state` (positions, velocities in original order) replaces the
    scene's initial state.  None when the reference's sources were not
    available to build it."""
    import oracle

    if oracle.ref_cuda_lib() is None:
        return None
    rparams = reference_cuda_params(bp, scene, params)
    ref = oracle.RefCudaSolver(scene, rparams)
    try:
        if state is not None:
            ref.set_state(*state)
        t0 = time.perf_counter()
        for _ in range(warmup):
            ref.update(SUBSTEPS, DT, ITERATIONS)
        ref.get(oracle.F_X)  # synchronises
        per = (time.perf_counter() - t0) / max(warmup, 1)
        k = max(1, min(steps, int(60.0 / max(per, 1e-6))))  # at most about a minute
        ms = ref.time_updates(k, SUBSTEPS, DT, ITERATIONS, flush.data_ptr(), flush.numel())
        x = ref.get(oracle.F_X)
        finite = bool(np.isfinite(x).all())
    finally:
        ref.close()
    n = scene.num_particles
    return {"value": n * SUBSTEPS * k / (ms / 1e3), "unit": "particle-substeps/s", "ms_per_step": ms / k,
            "steps": k, "warmup": warmup, "state_finite": finite, "stage_mask": int(rparams.stage_mask),
            "kind": "the reference's kernel headers (kernel/*.cuh) built unmodified for sm_103a, 128-thread "
                    "launches on the legacy default stream, toolkit CUB radix sort, stage order of "
                    "ParticleSolver::update with the constraint and wind blocks enabled"}


def run_batch(bp, torch, stream, flush, steps, warmup, seed=0):
    """The batched ensemble (256 scenes in one solver, its walk variant
    chosen by the autotuner after the warm-up) against looping the plain
    single-scene solver (default parameters) over the same scenes on the same
    stream."""
    scenes = bp.scenes.dam_break_ensemble(seed=seed)
    n = sum(s.num_particles for s in scenes)
    batch = bp.BatchSolver(scenes, stream=stream.cuda_stream)
    singles = [bp.ParticleSolver(s, stream=stream.cuda_stream) for s in scenes]
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            batch.update(SUBSTEPS, DT, ITERATIONS)
            for g in singles:
                g.update(SUBSTEPS, DT, ITERATIONS)
        tuned, trial_ms = batch.autotune(SUBSTEPS, DT, ITERATIONS)
        batch_shape = (batch.params.scan_block, batch.params.scan_persistent)
        batch.update(SUBSTEPS, DT, ITERATIONS)  # the chosen variant's graph, captured outside the timing
        for g in singles:
            g.update(SUBSTEPS, DT, ITERATIONS)
        launches_batch = batch.last_launch_count()
        launches_loop = sum(g.last_launch_count() for g in singles)
        ms_batch = timed_steps(torch, stream, flush, steps, lambda: batch.update(SUBSTEPS, DT, ITERATIONS))
        ms_loop = timed_steps(torch, stream, flush, steps,
                              lambda: [g.update(SUBSTEPS, DT, ITERATIONS) for g in singles])
    errors = batch.device_errors()
    batch.close()
    for g in singles:
        g.close()
    units = float(n) * SUBSTEPS * steps
    return {"workload": workload_name("batch", n), "scenes": len(scenes), "particles": n,
            "value": units / (ms_batch / 1e3), "loop_value": units / (ms_loop / 1e3),
            "batched_vs_loop": ms_loop / ms_batch, "ms_per_step": ms_batch / steps,
            "loop_ms_per_step": ms_loop / steps, "launches_per_step": launches_batch,
            "loop_launches_per_step": launches_loop, "device_errors": errors, "steps": steps,
            "autotune": {"walk_options": tuned, "scan_block": int(batch_shape[0]),
                         "scan_persistent": int(batch_shape[1]), "trial_ms": [round(t, 3) for t in trial_ms]}}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_throughput(torch, local_time, units_per_rank, world, device="cuda"):
    """Whole-job throughput of `world` replicas (each rank advances its own
    scene; no collective on the data path): every rank's units over the
    slowest rank's time (the maximum over ranks).  Returns (value, max time);
    times in seconds or milliseconds, value per the same unit."""
    t = torch.tensor([float(local_time)], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    t_max = float(t.item())
    return float(units_per_rank) * world / t_max, t_max


def profile_summary(kernel: str, workload: str):
    """The committed ncu summary of `kernel` for this workload: the early-frame
    capture where there is one (the timed frames are early ones), else the
    late-frame capture, else the 1,048,576-particle fluid capture.  Returns
    (text, file)."""
    name = kernel.replace("launch_", "k_")
    for fname in (f"{name}_{workload}_early.md", f"{name}_{workload}_late.md", f"{name}_fluid_1048576.md"):
        p = REPO / "profiles" / fname
        if p.exists():
            return p.read_text(), fname
    return None, None


def traffic_for(kernel: str, n: int, workload: str):
    """DRAM bytes per launch of `kernel` from its ncu summary, scaled to n
    particles (the traffic grows with the particle count)."""
    import re

    text, _ = profile_summary(kernel, workload)
    if text:
        t = re.search(r"DRAM traffic of the launch: ([0-9.]+) MB", text)
        parts = re.search(r"Particles: ([0-9]+)", text)
        if t and parts:
            return float(t.group(1)) * 1e6 * n / float(parts.group(1))
    return None


def issue_for(kernel: str, workload: str):
    """The scan kernels are bound by instruction issue, not by HBM: issue-slot
    use and active lanes per warp instruction from the same ncu summary."""
    import re

    text, fname = profile_summary(kernel, workload)
    if not text:
        return None
    busy = re.search(r"\| issue slots busy \| ([0-9.]+) %", text)
    lanes = re.search(r"\| active threads per warp instruction \(of 32\) \| ([0-9.]+)", text)
    if not (busy and lanes):
        return None
    return {"issue_slots_busy": round(float(busy.group(1)) / 100.0, 3),
            "active_lanes_of_32": float(lanes.group(1)), "source": "profiles/" + fname}


def workload_config(args, n, params, world):
    """The config object both arms print (same keys, same values)."""
    return {"workload": workload_name(args.workload, n), "particles": n, "substeps": SUBSTEPS,
            "iterations": ITERATIONS, "dt": DT, "mode": "reference",
            "grid": ("one grid per scene (16^3..64^3 cells), cell = h = 0.2" if args.workload == "batch"
                     else f"{params.grid_dim}^3 cells, cell = h = 0.2"),
            "neighbor_skin": float(params.neighbor_skin), "mass_scaling_k": float(params.mass_scaling_k),
            "stage_mask": int(params.stage_mask),
            "l2": "flushed (256 MB write) before every timed step", "parallelism": f"replicas x{world}"}


def run_ours(args):
    import torch

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import __graft_entry__ as entry

    entry.build()
    bp = entry.load_package()
    stream = torch.cuda.Stream()

    def tuned(p):
        if args.skin is not None:
            p.neighbor_skin = args.skin
        if args.no_stage:
            p.walk_options |= bp.abi.BP_WALK_NO_STAGING
        if args.no_split:
            p.walk_options |= bp.abi.BP_WALK_NO_SPLIT
        if args.no_lists:
            p.walk_options |= bp.abi.BP_WALK_NO_LISTS
        if args.contact_culling:
            p.walk_options &= ~bp.abi.BP_WALK_NO_CONTACT_CULLING
        if args.no_planes:
            p.walk_options |= bp.abi.BP_WALK_NO_PLANES
        return p

    if args.workload == "batch":
        scenes = bp.scenes.dam_break_ensemble(seed=rank)
        solver = bp.BatchSolver(scenes, [tuned(bp.make_params(s)) for s in scenes], stream=stream.cuda_stream)
        params = solver.params
        n = solver.n
    else:
        scene = build_scene(bp.scenes, args.workload, seed=rank)
        if args.load_state:  # continue a saved run (positions, velocities in original order)
            z = np.load(args.load_state)
            scene.positions, scene.velocities = z["x"].astype(np.float32), z["v"].astype(np.float32)
        n = scene.num_particles
        params = tuned(workload_params(bp, args.workload, scene))
        solver = bp.ParticleSolver(scene, params, stream=stream.cuda_stream)

    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            solver.update(SUBSTEPS, DT, ITERATIONS)
        tuned_walk = None
        if not (args.no_autotune or args.no_stage or args.no_split or args.no_lists):
            # keeps the fastest (bit-identical) walk variant
            opt, trial_ms = solver.autotune(SUBSTEPS, DT, ITERATIONS)
            tuned_walk = {"walk_options": opt, "scan_block": int(solver.params.scan_block),
                          "scan_persistent": int(solver.params.scan_persistent),
                          "trial_ms": [round(t, 3) for t in trial_ms]}
        stream.synchronize()
        launches_per_step = solver.last_launch_count()
        # the state the timed frames start from, for the end-to-end replay
        x_start = torch.from_numpy(solver.positions()).pin_memory()
        v_start = torch.from_numpy(solver.velocities()).pin_memory()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clocks:
            for k in range(args.steps):
                flush.fill_(k & 0xFF)  # evict the state from L2 between timed steps
                starts[k].record(stream)
                solver.update(SUBSTEPS, DT, ITERATIONS)
                ends[k].record(stream)
            torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    if args.save_state and rank == 0:
        np.savez(args.save_state, x=solver.positions(), v=solver.velocities())
    units = float(n) * SUBSTEPS * args.steps  # per rank
    value, ms_max = replica_throughput(torch, ms / 1e3, units, world)
    ms_max *= 1e3

    # end to end through the C ABI with host buffers: the same frames again,
    # each one's state uploaded from pinned host memory and its result
    # (positions and velocities, the next frame's input) read back
    import ctypes as C

    lib = solver.lib
    fp = C.POINTER(C.c_float)
    xs, vs = C.cast(x_start.data_ptr(), fp), C.cast(v_start.data_ptr(), fp)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bp.abi.check(lib, lib.bp_solver_set_state(solver.handle, xs, vs, bp.abi.BP_ORDER_ORIGINAL))
        solver.update(SUBSTEPS, DT, ITERATIONS)
        bp.abi.check(lib, lib.bp_solver_copy_positions(solver.handle, xs, bp.abi.BP_ORDER_ORIGINAL))
        bp.abi.check(lib, lib.bp_solver_copy_velocities(solver.handle, vs, bp.abi.BP_ORDER_ORIGINAL))
    e2e_s = time.perf_counter() - t0
    e2e_value, _ = replica_throughput(torch, e2e_s, units, world)

    roofline, stages, step_ms_total = kernel_roofline(torch, solver, n, args.workload, flush, value)
    walks = solver.walk_stats(SUBSTEPS, DT, ITERATIONS)
    device_errors = solver.device_errors()  # non-finite state anywhere in the run
    solver.close()
    reference_cuda = None
    if rank == 0 and args.workload != "batch" and not args.no_reference_cuda:
        ref_scene = build_scene(bp.scenes, args.workload, seed=0)
        reference_cuda = run_reference_cuda(bp, torch, ref_scene, workload_params(bp, args.workload, ref_scene),
                                            args.steps, args.warmup, flush)
        if reference_cuda is not None:
            reference_cuda["ours_over_reference"] = value / reference_cuda["value"]
    samples = None
    if rank == 0 and args.workload == "mixed" and not args.no_samples:
        samples = run_samples(bp, torch, stream, flush, local, args)
    batched = None
    if args.workload == "batch" or (args.workload == "mixed" and not args.no_batch):
        # the ensemble against a loop of one solver per scene, 10 timed frames each
        batched = run_batch(bp, torch, stream, flush, steps=10, warmup=3, seed=rank)
    adjoint = None
    if args.workload == "mixed" and not args.no_adjoint:
        adjoint = run_adjoint(bp, torch, stream, check_gradients=rank == 0 and not args.no_gradient_check)

    result = None
    if rank == 0:
        cpu = None if args.no_cpu_baseline else cpu_baseline(args.workload)
        clk = clocks.summary()
        result = {
            "metric": "particle-substeps/s",
            "value": value,
            "unit": "particle-substeps/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (seeded lattice scenes, no dataset)",
            "config": dict(workload_config(args, n, params, world), walk_options=int(solver.params.walk_options),
                           autotune=tuned_walk),
            "e2e": {"value": e2e_value, "unit": "particle-substeps/s",
                    "h2d_bytes_per_step": int(2 * n * 12), "d2h_bytes_per_step": int(2 * n * 12)},
            "gpu_launches": int(launches_per_step * args.steps),
            "roofline": roofline,
            "stages_ms_per_step": stages,
            "profiled_ms_per_step": step_ms_total,
            "neighbor_walks": walks,
            "device_errors": device_errors,
            "cpu_baseline": cpu,
            "clocks": clk,
        }
        if reference_cuda is not None:
            result["reference_cuda"] = reference_cuda
        if samples is not None:
            result["workloads"] = samples
        if batched is not None:
            result["batched"] = batched
        if adjoint is not None:
            result["adjoint"] = adjoint
        print(json.dumps(result), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return result


def workload_overrides(abi, workload):
    """Parameter overrides of a workload on top of the reference's literals:
    the stage set of the shape-matching stress test (planes, contacts, shape
    matching).  The mixed scene runs without mass scaling: exp(2 y) at the
    cloth's and cubes' heights (8 to 12 m) makes the contacts diverge within
    120 frames."""
    if workload == "mixed":
        return {"mass_scaling_k": 0.0}
    if workload == "rigid":
        return {"stage_mask": abi.BP_STAGE_PLANES | abi.BP_STAGE_PARTICLE_COLLISION | abi.BP_STAGE_SHAPE_MATCHING}
    return {}


def workload_params(bp, workload, scene):
    """bp_params of a workload through the product library."""
    return bp.make_params(scene, **workload_overrides(bp.abi, workload))


def reference_cpu_solver(oracle, scene, params, threads):
    """The reference's step on the host: its own kernels compiled for the host
    (oracle/_ref/libbrassref.so, kind "reference") where they were built,
    else the C restatement (kind "port")."""
    if oracle.ref_lib() is not None:
        return oracle.RefSolver(scene, params, threads=threads), "reference"
    return oracle.OracleSolver(scene, params, threads=threads), "port"


def cpu_baseline(workload, warm_substeps=1, substeps=2):
    """The reference's step on all host cores, on a bounded sample: one frame
    (`substeps` substeps) of the same scene after `warm_substeps` warm-up
    substeps, timed on the wall clock."""
    import oracle

    threads = os.cpu_count() or 1
    scenes = oracle.scenes_module()
    scene = build_scene(scenes, workload, seed=0)
    params = oracle.reference_params(scene, **workload_overrides(oracle._abi(), workload))
    solver, kind = reference_cpu_solver(oracle, scene, params, threads)
    for _ in range(warm_substeps):  # first touch of the grid tables
        solver.update(1, DT / SUBSTEPS, ITERATIONS)
    t0 = time.perf_counter()
    for _ in range(substeps):
        solver.update(1, DT / SUBSTEPS, ITERATIONS)
    dt = time.perf_counter() - t0
    what = ("the reference's kernels compiled for the host (OpenMP over the launch index)" if kind == "reference"
            else "the C restatement of the reference's step")
    return {"value": scene.num_particles * substeps / dt, "unit": "particle-substeps/s", "cores": threads,
            "kind": kind, "sample": f"{substeps} substeps of the same scene ({scene.num_particles} particles) after "
                                    f"{warm_substeps} warm-up substep: {what}, {threads} OpenMP threads"}


def run_reference(args):
    """Reference arm: the reference's step on the host cores, rank 0 only.
    It loads no product code: the scene comes from the pure-Python builders,
    the parameters from the reference's literals (oracle.reference_params), and
    the step from the reference's own kernels compiled for the host, else the
    C restatement.  Same workload, frames and warm-up as the GPU arm: W
    untimed updates, then K timed updates of 2 substeps (capped in time)."""
    rank, world, _ = dist_info()
    if rank != 0:
        return None
    import oracle

    oracle.build_oracle()
    oracle.build_ref()  # no-op without the reference's sources
    threads = os.cpu_count() or 1
    scenes = oracle.scenes_module()
    scene = build_scene(scenes, args.workload, seed=0)
    params = oracle.reference_params(scene, **workload_overrides(oracle._abi(), args.workload))
    solver, kind = reference_cpu_solver(oracle, scene, params, threads)
    n = scene.num_particles
    for _ in range(args.warmup):
        solver.update(SUBSTEPS, DT, ITERATIONS)
    budget_s = 240.0
    t0 = time.perf_counter()
    done = 0
    for _ in range(args.steps):
        solver.update(SUBSTEPS, DT, ITERATIONS)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    value = n * SUBSTEPS * done / dt
    what = ("the reference's kernels compiled for the host (OpenMP over the launch index)" if kind == "reference"
            else "the C restatement of the reference's step")
    sample = (f"{done} timed updates of {SUBSTEPS} substeps (frames {args.warmup + 1}..{args.warmup + done}; "
              f"capped at {budget_s:.0f} s) of the same scene ({n} particles) after {args.warmup} warm-up updates: "
              f"{what}, {threads} OpenMP threads")
    result = {
        "impl": "reference",
        "metric": "particle-substeps/s",
        "value": value,
        "unit": "particle-substeps/s",
        "n_gpus": world,
        "steps": done,
        "warmup": args.warmup,
        "ms_per_step": dt * 1e3 / max(done, 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded lattice scenes, no dataset)",
        "config": workload_config(args, n, params, world),
        "cpu_baseline": {"value": value, "unit": "particle-substeps/s", "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": "particle-substeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(result), flush=True)
    return result


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["mixed", "fluid", "small", "batch", "rigid"], default="mixed")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--no-reference-cuda", action="store_true", help="skip timing the reference's CUDA step")
    ap.add_argument("--no-samples", action="store_true", help="skip the other configurations and regimes")
    ap.add_argument("--no-gradient-check", action="store_true",
                    help="skip the FP64 finite-difference check of the adjoint's gradients")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the forward+adjoint measurement")
    ap.add_argument("--save-state", default=None, help="after the timed steps, save the state (npz) here")
    ap.add_argument("--load-state", default=None, help="start from a state saved by --save-state")
    ap.add_argument("--skin", type=float, default=None, help="Verlet-list skin (fraction of h); 0 disables")
    ap.add_argument("--no-stage", action="store_true", help="read neighbours from global memory only")
    ap.add_argument("--no-split", action="store_true", help="evaluate pair terms as candidates are tested")
    ap.add_argument("--no-lists", action="store_true", help="post passes B and C walk their cells")
    ap.add_argument("--no-planes", action="store_true",
                    help="recording walks read the position records instead of the walk planes")
    ap.add_argument("--no-autotune", action="store_true", help="keep the walk options given instead of timing them")
    ap.add_argument("--contact-culling", action="store_true",
                    help="contact walks over only the cells a partner can be stored in (with --no-autotune)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
