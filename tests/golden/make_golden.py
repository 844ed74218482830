"""Generates the golden fixtures in this directory from the REFERENCE ITSELF.

The reference's own kernel headers (brasstower/kernel/*.cuh) are compiled for
the host through oracle/refshim (`make -C oracle ref`, needs the reference
checkout) and driven by oracle/ref_driver.cpp, single-threaded so every
scatter runs in a fixed order.  Outputs are written as small .npz files that
travel with the repository (the GPU machine has no reference checkout):

  grid_*.npz   positions -> cell ids, stable sorted order, cellStart/cellEnd
               of occupied cells, 27-cell neighbour counts
  step_*.npz   a scene (all arrays + parameters) and the state after
               `frames` calls of update(2 substeps, 1/60 s, 4 iterations)

kernel/bending.cuh:52 negates a temporary, which helper_math.h's unary minus
(a non-const reference) cannot bind; ref_driver.cpp adds an rvalue overload
so that the unmodified kernel compiles.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests"))

SCENE_ARRAYS = ["positions", "velocities", "masses", "phases", "group_ids", "planes", "distance_pairs",
                "distance_params", "faces", "rigid_ranges", "rigid_rest", "immovables", "bendings"]
SCENE_SCALARS = ["particle_radius", "kernel_radius", "cell_size", "grid_dim", "rest_density"]


def scene_to_dict(s, prefix="scene_"):
    out = {}
    for k in SCENE_ARRAYS:
        v = getattr(s, k)
        if v is not None:
            out[prefix + k] = np.asarray(v)
    for k in SCENE_SCALARS:
        out[prefix + k] = np.asarray(getattr(s, k))
    return out


def scene_from_npz(z, scenes_mod, prefix="scene_"):
    s = scenes_mod.Scene()
    for k in SCENE_ARRAYS:
        if prefix + k in z:
            setattr(s, k, np.array(z[prefix + k]))
        elif k == "velocities":
            s.velocities = None
    for k in SCENE_SCALARS:
        v = z[prefix + k].item()
        setattr(s, k, int(v) if k == "grid_dim" else float(v))
    return s


def grid_fixture(name, pos, cell, D, h):
    import oracle

    cid, scid, spid, cs, ce = oracle.grid_build("ref", pos, cell, D)
    occ = np.nonzero(cs >= 0)[0].astype(np.int32)
    counts = oracle.neighbor_counts("ref", pos[spid], cell, D, h, cs, ce)
    np.savez_compressed(HERE / name, positions=pos.astype(np.float32), cell=np.float32(cell), D=np.int32(D),
                        h=np.float32(h), cell_ids=cid, sorted_cell_ids=scid, sorted_particle_ids=spid,
                        occupied=occ, cell_start=cs[occ], cell_end=ce[occ], neighbor_counts=counts)
    print(f"{name}: N={len(pos)} D={D} occupied={len(occ)} max count={counts.max() if len(counts) else 0}")


def step_fixture(name, bp, scene, frames, mask=None):
    import oracle

    params = bp.make_params(scene)
    if mask is not None:
        params.stage_mask = mask
    r = oracle.RefSolver(scene, params, threads=1)
    out = scene_to_dict(scene)
    out["stage_mask"] = np.int32(params.stage_mask)
    out["frames"] = np.int32(frames)
    for f in range(frames):
        r.update(2, 1.0 / 60.0, 4)
        if f == 0:
            out["x1"] = r.positions()
            out["v1"] = r.velocities()
            out["to_orig1"] = r.get(oracle.F_TO_ORIG)
            out["sorted_cell1"] = r.get(oracle.F_SORTED_CELL)
            out["lambda1"] = r.get(oracle.F_LAMBDA)
            out["density1"] = r.get(oracle.F_DENSITY)
    out["x"] = r.positions()
    out["v"] = r.velocities()
    out["to_orig"] = r.get(oracle.F_TO_ORIG)
    if len(scene.rigid_ranges):
        out["rotations"] = r.get(oracle.F_ROT)
        out["cms"] = r.get(oracle.F_CM)
    np.savez_compressed(HERE / name, **out)
    print(f"{name}: N={scene.num_particles} frames={frames}")


def main():
    import __graft_entry__ as entry
    import oracle
    from conftest import cloth_bending_scene, fluid_scene, small_mixed_scene

    entry.build()
    if oracle.ref_lib() is None:
        raise SystemExit("the reference checkout is required to generate golden fixtures")
    bp = entry.load_package()
    rng = np.random.default_rng(2024)

    # grid: ragged N, negative coordinates, D = 32
    pos = rng.uniform(-3.0, 3.0, (3001, 3)).astype(np.float32)
    grid_fixture("grid_d32.npz", pos, 0.2, 32, 0.2)
    # grid: heavy aliasing of the table (D = 4) and many ties per cell
    pos = rng.uniform(0.0, 4.0, (777, 3)).astype(np.float32)
    grid_fixture("grid_d4_alias.npz", pos, 0.2, 4, 0.2)
    # grid: points exactly on cell faces, duplicates, one far outlier
    base = (rng.integers(-8, 8, (600, 3)) * np.float32(0.25)).astype(np.float32)
    base = np.concatenate([base, base[:50], np.array([[1000.0, -1000.0, 0.5]], np.float32)])
    grid_fixture("grid_faces_d16.npz", base, 0.25, 16, 0.25)
    # grid: the reference's own table size D = 512 (2^27 cells)
    pos = rng.uniform(-1.0, 1.0, (1500, 3)).astype(np.float32)
    grid_fixture("grid_d512.npz", pos, 0.115, 512, 0.115)
    # grid: a single particle
    grid_fixture("grid_single.npz", np.array([[0.3, -0.2, 0.1]], np.float32), 0.2, 8, 0.2)

    step_fixture("step_fluid.npz", bp, fluid_scene(bp, (10, 10, 10), seed=3, grid_dim=32), frames=10)
    step_fixture("step_mixed.npz", bp, small_mixed_scene(bp, seed=5), frames=10)
    s = small_mixed_scene(bp, seed=6)
    step_fixture("step_mixed_as_shipped.npz", bp, s, frames=3,
                 mask=bp.abi.BP_STAGE_PLANES | bp.abi.BP_STAGE_VORTICITY | bp.abi.BP_STAGE_AKINCI
                 | bp.abi.BP_STAGE_XSPH | bp.abi.BP_STAGE_FLUID)
    # dihedral bending (kernel/bending.cuh, compiled with an rvalue negation overload)
    step_fixture("step_cloth_bending.npz", bp, cloth_bending_scene(bp, seed=7), frames=10)


if __name__ == "__main__":
    main()
