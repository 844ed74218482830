/*
 * brasspan.h -- C ABI of the GB300-native unified particle solver step.
 *
 * This is the drop-in boundary for brass-pan's `ParticleSolver`
 * (brasstower/particlesolver.cuh).  Every entry point is plain C: opaque
 * handles, plain pointers and sizes, integer status codes, no exceptions and
 * no C++ or PyTorch types.  Each declaration names the reference interface it
 * replaces (file:line inside the brass-pan project).
 *
 * Memory: the solver owns its device memory (bp_solver_destroy frees it).
 * Arrays are kept in cell-sorted order between steps, exactly like the
 * reference keeps devPositions & co. permuted (particlesolver.cuh:758-764);
 * original ids map through bp_solver_query_* or bp_solver_copy_* with
 * BP_ORDER_ORIGINAL.
 *
 * Streams: each solver is bound to the CUDA stream given at creation (NULL =
 * legacy default stream, as the reference uses).  Calls on one solver are not
 * thread-safe; different solvers are independent.  bp_solver_update only
 * enqueues work (a CUDA graph replay after the first call of a given shape);
 * the copy / query / error entry points synchronise the stream.
 */
#ifndef BRASSPAN_H
#define BRASSPAN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BP_ABI_VERSION 1

typedef enum bp_status {
    BP_OK = 0,
    BP_ERR_INVALID_ARGUMENT = 1, /* NULL handle, negative count, bad id, ... */
    BP_ERR_CUDA = 2,             /* a CUDA runtime call failed */
    BP_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed */
    BP_ERR_CAPACITY = 4,         /* a size is beyond a documented limit */
    BP_ERR_DEVICE_CHECK = 5,     /* a device-side check fired during the last step */
    BP_ERR_NO_DEVICE = 6         /* no CUDA device visible */
} bp_status;

/* Bits of the device error word (bp_solver_device_errors). */
#define BP_DEVERR_NONFINITE 0x1u     /* a predicted position became NaN/Inf */
#define BP_DEVERR_RIGID_SIZE 0x2u    /* reserved */
#define BP_DEVERR_BAD_INDEX 0x4u     /* a constraint referenced an id outside [0, N) */

/* Parameter presets. */
typedef enum bp_mode {
    /* Reproduces the reference kernels as written, quirks included
     * (density over j >= i, precomputed lambda denominator, per-pair clamp,
     * Akinci spline inner branch, wind without a wind vector, ...). */
    BP_MODE_REFERENCE = 0,
    /* Textbook position-based fluids (Macklin & Mueller 2013): density over
     * all neighbours, lambda = -C / (sum |grad C|^2 + eps), s_corr active,
     * no per-pair clamp, wind relative to a wind vector. */
    BP_MODE_TEXTBOOK = 1
} bp_mode;

/* Stage switches (bp_params.stage_mask).  BP_STAGE_ALL is the reference's
 * update() with its commented-out constraint block (particlesolver.cuh:881-993)
 * and wind block (:838-858) enabled. */
#define BP_STAGE_PLANES 0x001
#define BP_STAGE_WIND 0x002
#define BP_STAGE_PARTICLE_COLLISION 0x004
#define BP_STAGE_FLUID 0x008
#define BP_STAGE_DISTANCE 0x010
#define BP_STAGE_SHAPE_MATCHING 0x020
#define BP_STAGE_IMMOVABLE 0x040
#define BP_STAGE_VORTICITY 0x080
#define BP_STAGE_AKINCI 0x100
#define BP_STAGE_XSPH 0x200
#define BP_STAGE_BENDING 0x400
#define BP_STAGE_ALL 0x7ff
/* The stages the reference's update() runs as shipped (only planes and the
 * velocity post-passes are live there). */
#define BP_STAGE_REFERENCE_AS_SHIPPED \
    (BP_STAGE_PLANES | BP_STAGE_VORTICITY | BP_STAGE_AKINCI | BP_STAGE_XSPH)

/* bp_params.walk_options (results are identical under every combination):
 * BP_WALK_NO_STAGING reads every neighbour from global memory instead of
 * staging each block's neighbourhood in shared memory; BP_WALK_NO_SPLIT
 * evaluates each pair term as its candidate is tested instead of testing a
 * chunk of candidates first and evaluating the pair terms of the hits;
 * BP_WALK_NO_LISTS makes the position pass and the second and third
 * velocity post passes walk their cells instead of reading the neighbour
 * lists that the lambda pass and the first post pass record;
 * BP_WALK_NO_ALIAS_CLASSES makes unstaged walks test every particle of a
 * table cell instead of only those of the real cell walked (a grid of D^3
 * cells wraps space, so one table cell holds every real cell D cells apart;
 * the split is kept for grids of at most 2^21 cells and used in a substep
 * while at least 1/32 of the particles share a cell with another real cell's
 * and no particle has moved (D - 2) cells - h from where it was hashed);
 * BP_WALK_NO_FUSION runs each iteration's plane collision and the final
 * velocity update and commit as launches of their own, instead of fused into
 * the reorder (iteration 0's planes) and the position pass's epilogue (the
 * next iteration's planes, or the commit after the last iteration);
 * BP_WALK_NO_CONTACT_CULLING makes the particle-contact walks visit all 27
 * cells instead of only the cells a contact partner can be stored in (from
 * a bound on every particle's displacement since its cell was hashed);
 * BP_WALK_NO_PLANES makes the recording walks of the lambda pass and the
 * first post pass (unstaged, split) read each candidate's position record
 * instead of the walk planes, copies of x, y, z and the phase in separate
 * arrays written just before those passes, from which four candidates are
 * tested per three vector loads with paired fp32 arithmetic and each chunk
 * of 32 candidates' hits is appended to the list a record at a time. */
#define BP_WALK_NO_STAGING 0x1
#define BP_WALK_NO_SPLIT 0x2
#define BP_WALK_NO_LISTS 0x4
#define BP_WALK_NO_ALIAS_CLASSES 0x8
#define BP_WALK_NO_FUSION 0x10
#define BP_WALK_NO_CONTACT_CULLING 0x20
#define BP_WALK_NO_PLANES 0x40

/* Every literal of the reference's step as a field.  bp_params_init fills the
 * reference's values; comments give the reference location of each. */
typedef struct bp_params {
    int32_t mode;                /* bp_mode */
    int32_t stage_mask;          /* BP_STAGE_* */
    float gravity[3];            /* (0,-9.8,0), added as g*dt*dt to the prediction (particlesolver.cuh:56) */
    float particle_radius;       /* solid radius: planes and contacts (scene.h:500) */
    float kernel_radius;         /* SPH smoothing length h (fluid.cuh:11) */
    float cell_size;             /* hash cell edge; the reference uses 2.3*radius == h (particlesolver.cuh:221) */
    int32_t grid_dim;            /* D, power of two in [4, 512]: D^3 cells (particlesolver.cuh:222 uses 512) */
    float rest_density;          /* rho0 (scene.h OldSceneFormat::fluidRestDensity) */
    float solid_density_scale;   /* 2.0 (particlesolver.cuh:909) */
    float lambda_denominator;    /* 15000, reference mode (fluid.cuh:153) */
    float relaxation;            /* epsilon of the exact lambda, textbook mode (fluid.cuh:155) */
    float scorr_k;               /* 0.0001 (particlesolver.cuh:926) */
    int32_t scorr_n;             /* 4 (particlesolver.cuh:927) */
    float scorr_dq;              /* s_corr reference distance as a fraction of h: 0.03 (fluid.cuh:208) */
    float delta_clamp;           /* per-pair |delta p| clamp: 5.0 (fluid.cuh:214); <= 0 disables */
    float vorticity_eps;         /* 0.001 (particlesolver.cuh:1017) */
    float surface_tension;       /* Akinci gamma 0.5 (particlesolver.cuh:1043) */
    float xsph_c;                /* 0.0002 (particlesolver.cuh:1055) */
    float friction_static;       /* 0.5 (cubrasstower.cuh:18) */
    float friction_dynamic;      /* 0.0 (cubrasstower.cuh:19) */
    float mass_scaling_k;        /* 2 (cubrasstower.cuh:20) */
    float wind_velocity[3];      /* textbook mode only: the wind vector */
    float wind_drag;             /* 10 (wind.cuh:40) */
    float wind_lift;             /* 100 (wind.cuh:43) */
    int32_t rotation_iterations; /* 20 (shapematching.cuh:72) */
    float neighbor_skin;         /* skin of the per-substep Verlet lists, as a fraction of h
                                    (0 disables them; results are identical either way): 0 */
    int32_t walk_options;        /* BP_WALK_* tuning switches of the neighbour walks:
                                    BP_WALK_NO_STAGING | BP_WALK_NO_CONTACT_CULLING */
    float bending_stiffness;     /* 0.8 (bending.cuh:71) */
    /* Launch shape of the neighbour-scan kernels when they do not stage
     * (BP_WALK_NO_STAGING; results are identical under every shape):
     * threads per CTA (0 = 256; 64, 128 or 256), and persistent launches
     * (1: no more CTAs than fit on the GPU at once, each looping over the
     * 256-, 128- or 64-particle tiles).  bp_solver_autotune picks them. */
    int32_t scan_block;          /* 0 */
    int32_t scan_persistent;     /* 0 */
    int32_t reserved[3];
} bp_params;

/* Fills `p` with the reference's literals for a scene of the given particle
 * radius (h = cell = 2.3 * radius, D = 512, rho0 = 1200 as initFluidScene). */
void bp_params_init(bp_params *p, float particle_radius);

/* Scene description in original particle order (host pointers, copied at
 * creation).  Replaces the reference's `Scene` vectors (scene.h:455-535) and
 * the OldSceneFormat objects (scene.h:39-435). */
typedef struct bp_scene_desc {
    int32_t num_particles;
    const float *positions;            /* [N][3] */
    const float *velocities;           /* [N][3] or NULL for zero */
    const float *masses;               /* [N], > 0 */
    const int32_t *phases;             /* [N]: < 0 fluid, > 0 solid (never 0) */
    const int32_t *group_ids;          /* [N] or NULL (render grouping only) */
    int32_t num_planes;
    const float *planes;               /* [P][6]: origin xyz, unit normal xyz */
    int32_t num_distance_constraints;
    const int32_t *distance_pairs;     /* [M][2] original ids */
    const float *distance_params;      /* [M][2]: rest length, stiffness */
    int32_t num_wind_faces;
    const int32_t *wind_faces;         /* [F][3] original ids */
    int32_t num_rigid_bodies;
    const int32_t *rigid_ranges;       /* [B][2]: [first, last+1) original ids */
    const float *rigid_rest_positions; /* [N][3] by original id; each body's rest shape has its centre at 0 */
    int32_t num_immovables;
    const int32_t *immovables;         /* [K] original ids */
    int32_t num_bendings;              /* dihedral bending constraints (kernel/bending.cuh) */
    const int32_t *bendings;           /* [Q][4] original ids: hinge edge (0, 1), wings 2 and 3; rest: flat */
} bp_scene_desc;

typedef struct bp_solver bp_solver;

/* ParticleSolver(const shared_ptr<Scene>&) / ParticleSolver(shared_ptr<OldSceneFormat>)
 * (particlesolver.cuh:148-215, :218-342).  `stream` is a cudaStream_t or NULL. */
bp_status bp_solver_create(const bp_scene_desc *scene, const bp_params *params, void *stream,
                           bp_solver **out);

/* The reference never frees its buffers ("TODO:: implement object's destroyer",
 * particlesolver.cuh:1074); this releases everything the solver owns. */
bp_status bp_solver_destroy(bp_solver *s);

/* ParticleSolver::update(numSubTimeStep, deltaTime, pickedOriginalParticleId,
 * pickedParticlePosition, pickedParticleVelocity) (particlesolver.cuh:772-1072),
 * with the solver-iteration count, hard-coded to 2 there (:862), as a
 * parameter.  picked_original_id < 0 disables picking; picked_* may then be NULL. */
bp_status bp_solver_update(bp_solver *s, int32_t num_substeps, float dt, int32_t iterations,
                           int32_t picked_original_id, const float *picked_position,
                           const float *picked_velocity);

/* update() without picking. */
bp_status bp_solver_step(bp_solver *s, float dt, int32_t num_substeps, int32_t iterations);

/* Replaces the parameters (takes effect at the next update). */
bp_status bp_solver_set_params(bp_solver *s, const bp_params *params);

/* Copies the solver's current parameters (for instance the walk options and
 * scan launch shape bp_solver_autotune chose).  No counterpart in the
 * reference, whose parameters are literals. */
bp_status bp_solver_get_params(const bp_solver *s, bp_params *out);

/* queryOriginalParticleId / queryNewParticleId (particlesolver.cuh:352-366). */
bp_status bp_solver_query_original_particle_id(bp_solver *s, int32_t sorted_index, int32_t *out);
bp_status bp_solver_query_new_particle_id(bp_solver *s, int32_t original_id, int32_t *out);

/* getParticlePosition(sorted index) (particlesolver.cuh:378-386). */
bp_status bp_solver_get_particle_position(bp_solver *s, int32_t sorted_index, float out_xyz[3]);

typedef enum bp_order { BP_ORDER_SORTED = 0, BP_ORDER_ORIGINAL = 1 } bp_order;

/* Host copies of the state ([N][3] floats), synchronising the solver's stream. */
bp_status bp_solver_copy_positions(bp_solver *s, float *host_xyz, int32_t order);
bp_status bp_solver_copy_velocities(bp_solver *s, float *host_xyz, int32_t order);
/* Overwrites positions and velocities (host [N][3], either may be NULL).
 * The cell-sorted order stays as it is; the reference's density sums depend
 * on that order, so a run continued from set_state need not repeat the bits
 * of one that was never interrupted (bp_solver_snapshot_* does). */
bp_status bp_solver_set_state(bp_solver *s, const float *host_positions,
                              const float *host_velocities, int32_t order);

/* Checkpoint / resume; no counterpart in the reference.  A snapshot is one
 * host byte buffer holding everything a later update or query reads: the
 * committed and predicted state in its cell-sorted order, the id maps, the
 * grid, lambda and density, rigid rotations and centres, the device error
 * word.  Loading it into a solver created from the same scene (same particle
 * count, grid and rigid bodies; checked) continues the run bit for bit.
 * Parameters are not part of it.  Neither call is allowed while a tape records. */
bp_status bp_solver_snapshot_size(bp_solver *s, size_t *bytes);
bp_status bp_solver_snapshot_save(bp_solver *s, void *host, size_t bytes);
bp_status bp_solver_snapshot_load(bp_solver *s, const void *host, size_t bytes);

typedef enum bp_field {
    BP_FIELD_POSITIONS = 0,      /* float4 [N]: committed x, w = mass */
    BP_FIELD_NEW_POSITIONS = 1,  /* float4 [N]: predicted p, w = phase (int bits) */
    BP_FIELD_VELOCITIES = 2,     /* float4 [N] */
    BP_FIELD_MAP_TO_ORIGINAL = 3,/* int32 [N]: sorted index -> original id */
    BP_FIELD_MAP_TO_NEW = 4,     /* int32 [N]: original id -> sorted index */
    BP_FIELD_LAMBDAS = 5,        /* float [N] */
    BP_FIELD_DENSITIES = 6,      /* float [N] */
    BP_FIELD_SORTED_CELL_IDS = 7,/* int32 [N] */
    BP_FIELD_CELL_OFFSETS = 8,   /* int32 [D^3+1]: first sorted index of each cell */
    BP_FIELD_RIGID_ROTATIONS = 9,/* float4 [B] quaternion (x,y,z,w) */
    BP_FIELD_RIGID_CMS = 10,     /* float4 [B] */
    BP_FIELD_INV_SCALED_MASSES = 11, /* float [N] */
    BP_FIELD_COUNT = 12
} bp_field;

/* Device pointer and byte size of a field (valid until the next update;
 * fields are swapped between buffers inside update, like the reference's
 * std::swap calls at particlesolver.cuh:758-764,1048,1060). */
bp_status bp_solver_field(bp_solver *s, int32_t field, void **device_ptr, size_t *bytes);
/* Synchronous host copy of a whole field. */
bp_status bp_solver_copy_field(bp_solver *s, int32_t field, void *host_dst, size_t bytes);

/* Headless stand-in for the render hand-off mapParticleInfos (main.cu:273-282):
 * writes N records {float x, y, z; int32 phase} (16 bytes each, sorted order)
 * into a caller-owned device buffer, on the solver's stream. */
bp_status bp_solver_pack_particle_infos(bp_solver *s, void *device_out);

/* Reads and clears the device error word (BP_DEVERR_* bits). */
bp_status bp_solver_device_errors(bp_solver *s, uint32_t *out_bits);

/* Number of kernels the last bp_solver_update enqueued. */
bp_status bp_solver_last_launch_count(bp_solver *s, int64_t *out);

/* Per-stage device time of one update (no graph; a CUDA event after every
 * kernel on the solver's stream).  Replaces the reference's only timing, the
 * ms/frame in the window title (main.cu:418-428).  Writes up to `capacity`
 * entries, one per kernel name, and the number of distinct names to *count.
 * The update is real: it advances the state like bp_solver_update. */
typedef struct bp_stage_time {
    char name[48];
    int32_t launches;
    float total_ms;
} bp_stage_time;
bp_status bp_solver_profile(bp_solver *s, int32_t num_substeps, float dt, int32_t iterations,
                            int32_t capacity, bp_stage_time *out, int32_t *count);

/* One real update that also counts the neighbour walks of every scan pass:
 * out_walks[0] walks over the per-substep Verlet lists; 27-cell walks
 * because [1] no list was built for the particle (lists are off, the pass
 * builds them, its column runs wrap around the table, or its list held more
 * than 256 candidates), [2] the particle left the cell its list was built
 * for, [3] it or a particle stored in its 27 cells moved more than half the
 * skin; [4] of the cell walks, those restricted to the alias classes. */
bp_status bp_solver_walk_stats(bp_solver *s, int32_t num_substeps, float dt, int32_t iterations,
                               uint64_t out_walks[5]);

/* Picks the fastest neighbour-walk variant and scan launch shape for this
 * solver's scene and step configuration (all give identical results): each
 * candidate runs one update from the current state, timed with CUDA events,
 * and the state is put back after every trial.  First the 8 combinations of
 * the three BP_WALK_NO_* bits at the default launch shape, in the order 0,
 * NO_STAGING, NO_SPLIT, NO_LISTS, NO_STAGING|NO_SPLIT, NO_STAGING|NO_LISTS,
 * NO_SPLIT|NO_LISTS, all three; then, when the fastest of them does not
 * stage, its unstaged scans with 128 and with 64 threads per CTA and with
 * persistent 256-thread CTAs (bp_params.scan_block, .scan_persistent); then
 * the fastest so far without iteration fusion (BP_WALK_NO_FUSION), and, in a
 * scene with particle contacts, with the contact walks' cell culling (without
 * BP_WALK_NO_CONTACT_CULLING), each kept only when more than 1 % faster.  The
 * choice is kept in the solver's parameters and its walk options written to
 * *out_walk_options; out_ms (or NULL) receives the 13 trial times in that
 * order (0 for a trial not run).  No counterpart in the reference. */
bp_status bp_solver_autotune(bp_solver *s, int32_t num_substeps, float dt, int32_t iterations,
                             int32_t *out_walk_options, float *out_ms);

/* ---- Differentiable rollouts ------------------------------------------------
 * No counterpart in the reference.  bp_solver_tape_begin starts recording the
 * following bp_solver_update calls (no picking); the state is checkpointed at
 * the start of an update once `checkpoint_every` substeps have passed since
 * the last checkpoint.  bp_solver_backward then returns the gradient of a
 * scalar loss L(x_T, v_T) of the final state with respect to the state when
 * recording began and to parameters, given dL/dx_T and dL/dv_T ([N][3] host
 * arrays in original order; either may be NULL for zero).  It re-runs the
 * substeps between checkpoints (the neighbour sets of the adjoint are those
 * of the re-run forward pass) and restores the solver's state afterwards, so
 * stepping may continue; the tape stays open until bp_solver_tape_end.
 *
 * Stages with an adjoint: planes, wind, particle-particle contacts with
 * friction, distance constraints, dihedral bending, shape matching (the
 * extracted rotation differentiated at its fixed point), immovables, the
 * velocity update, the fluid density / lambda / position correction (both
 * modes), vorticity confinement, Akinci tension, XSPH and picking (the
 * picked particle's gradient is 0 before each point where it is set). */
typedef struct bp_gradients {
    float *positions;            /* [N][3] dL/dx at tape begin, original order, or NULL */
    float *velocities;           /* [N][3] dL/dv at tape begin, or NULL */
    float *wind_velocity;        /* [3] dL/d wind_velocity (textbook wind), or NULL */
    float *distance_stiffness;   /* [M] dL/d stiffness of each distance constraint, or NULL */
    float *distance_rest_length; /* [M] dL/d rest length, or NULL */
} bp_gradients;
bp_status bp_solver_tape_begin(bp_solver *s, int32_t checkpoint_every);
bp_status bp_solver_backward(bp_solver *s, const float *grad_positions, const float *grad_velocities,
                             bp_gradients *out);
bp_status bp_solver_tape_end(bp_solver *s);

/* ---- Batched ensembles ----------------------------------------------------
 * No counterpart in the reference, which steps one scene per solver.  Many
 * independent scenes advance together, one kernel launch per stage over all
 * of their particles: each scene keeps its own hash grid (params[k].grid_dim)
 * inside one shared key space, its own rest density, gravity and planes, and
 * every other parameter is shared (params[k] may differ from params[0] only
 * in rest_density, gravity and grid_dim; Verlet lists are not available).
 * Scene k's particles, stepped in a batch, follow exactly the trajectory a
 * solver of scene k alone gives.
 *
 * The batch is a bp_solver: its particles are the scenes' particles in scene
 * order (scene k's particle i has original id first_k + i, first_k from
 * bp_batch_scene_range), and every bp_solver_* entry point applies to it.
 * Capacity: 2^28 particles, 2^30 grid cells in total. */
bp_status bp_batch_create(int32_t num_scenes, const bp_scene_desc *scenes, const bp_params *params,
                          void *stream, bp_solver **out);
/* bp_solver_step of a batch (BP_ERR_INVALID_ARGUMENT for a single-scene solver). */
bp_status bp_batch_step(bp_solver *batch, float dt, int32_t num_substeps, int32_t iterations);
/* First original id and particle count of scene `scene`. */
bp_status bp_batch_scene_range(const bp_solver *batch, int32_t scene, int32_t *first, int32_t *count);

/* ---- Stand-alone hash grid on caller-owned device buffers ---------------
 * Replaces updateGrid() (particlesolver.cuh:712-765): updateGridId
 * (kernel/grid.cuh:30-47), the CUB stable radix sort (particlesolver.cuh:721-738)
 * and findStartEndId (kernel/grid.cuh:70-99).  positions are [N][3] floats.
 * cell_start/cell_end hold D^3 int32 each and, as in the reference, must be
 * -1 everywhere before the call (set once, then restored by bp_grid_reset);
 * only the entries of occupied cells are written. */
bp_status bp_grid_workspace_size(int32_t num_particles, int32_t grid_dim, size_t *bytes);
bp_status bp_grid_build(void *stream, int32_t num_particles, const float *d_positions,
                        float cell_size, int32_t grid_dim, int32_t *d_cell_ids,
                        int32_t *d_sorted_cell_ids, int32_t *d_sorted_particle_ids,
                        int32_t *d_cell_start, int32_t *d_cell_end, void *d_workspace,
                        size_t workspace_bytes);
/* resetStartEndId (kernel/grid.cuh:101-132). */
bp_status bp_grid_reset(void *stream, int32_t num_particles, const int32_t *d_sorted_cell_ids,
                        int32_t *d_cell_start, int32_t *d_cell_end);

/* bp_grid_build without a workspace and without any allocation.  This entry
 * point has no counterpart in the reference.  It is for callers that cannot
 * call cudaMalloc when they need a grid: a plug-in inside a host application
 * that owns all device memory through its own pools, a real-time loop whose
 * budget forbids allocation after start-up, or code that must not
 * synchronise the device, as cudaMalloc and cudaFree may do.
 *
 * The sort's scratch is a fixed 4.2 MB array in the library's device memory,
 * held on every GPU that loads the library until the process exits, so
 * num_particles is at most 262144; larger inputs return BP_ERR_CAPACITY.
 * Inputs, outputs and their contract are those of bp_grid_build (cell_start /
 * cell_end -1 before the call; grid_dim a power of two in 4..1024).
 *
 * The first call on a device, with that device current, looks up the array's
 * address on that device; make that first call before any stream capture.
 * The address is kept for the rest of the process: after cudaDeviceReset (or
 * any other teardown of the device's primary context) it no longer points at
 * the array, so do not call this entry point in a process that has reset the
 * device since its first call there.
 * All calls on a device share the one array: calls whose work overlaps on the
 * GPU (on different streams, or from different threads without ordering)
 * race and give wrong results.  Order them on one stream. */
bp_status bp_grid_build_static(void *stream, int32_t num_particles, const float *d_positions,
                               float cell_size, int32_t grid_dim, int32_t *d_cell_ids,
                               int32_t *d_sorted_cell_ids, int32_t *d_sorted_particle_ids,
                               int32_t *d_cell_start, int32_t *d_cell_end);

/* Neighbour counts in the reference's 27-cell walk (the loop structure of
 * kernel/fluid.cuh:104-141): for each particle i of the cell-sorted positions
 * [N][3], the number of j (i itself included) stored in the 27 cells around
 * the cell of p_i with |p_i - p_j|^2 <= h^2.  start/end as from bp_grid_build. */
bp_status bp_grid_neighbor_counts(void *stream, int32_t num_particles, const float *d_sorted_positions,
                                  float cell_size, int32_t grid_dim, float kernel_radius,
                                  const int32_t *d_cell_start, const int32_t *d_cell_end,
                                  int32_t *d_counts);

/* Last error message of this thread ("" if none). */
const char *bp_last_error_string(void);

/* ABI version and build description. */
int32_t bp_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* BRASSPAN_H */
