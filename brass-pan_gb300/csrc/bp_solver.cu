// bp_solver.cu -- the solver handle, step orchestration and the C ABI.
//
// bp_solver_update replays the stage order of ParticleSolver::update
// (brasstower/particlesolver.cuh:787-1063) with the commented constraint
// block (:881-993) and wind block (:838-858) enabled and the iteration count
// as a parameter.  The whole call is captured once into a CUDA graph per
// (substeps, iterations, dt, parameters) and replayed afterwards.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "bp_solver_state.h"

using namespace bp;

namespace {

thread_local std::string g_err;

bp_status fail(bp_status st, const std::string &msg)
{
    g_err = msg;
    return st;
}

// Inside create_solver: a failure frees the half-built solver first.
#define BP_CUDA_BAIL(call)                                                                     \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return bail(fail(e_ == cudaErrorMemoryAllocation ? BP_ERR_OUT_OF_MEMORY : BP_ERR_CUDA, \
                             std::string(#call) + ": " + cudaGetErrorString(e_)));             \
    } while (0)

#define BP_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(e_ == cudaErrorMemoryAllocation ? BP_ERR_OUT_OF_MEMORY : BP_ERR_CUDA,  \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                   \
    } while (0)

bool is_pow2(int d) { return d > 0 && (d & (d - 1)) == 0; }

}  // namespace

// The message bp_last_error_string returns, for entry points in other files.
void bp::set_last_error(const char *msg) { g_err = msg; }

extern "C" void bp_params_init(bp_params *p, float r)
{
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->mode = BP_MODE_REFERENCE;
    p->stage_mask = BP_STAGE_ALL;
    p->gravity[0] = 0.f;
    p->gravity[1] = -9.8f;
    p->gravity[2] = 0.f;
    p->particle_radius = r;
    p->kernel_radius = 2.3f * r;
    p->cell_size = r * 2.3f;
    p->grid_dim = 512;
    p->rest_density = 1200.f;
    p->solid_density_scale = 2.0f;
    p->lambda_denominator = 15000.0f;
    p->relaxation = 300.0f;
    p->scorr_k = 0.0001f;
    p->scorr_n = 4;
    p->scorr_dq = 0.03f;
    p->delta_clamp = 5.0f;
    p->vorticity_eps = 0.001f;
    p->surface_tension = 0.5f;
    p->xsph_c = 0.0002f;
    p->friction_static = 0.5f;
    p->friction_dynamic = 0.0f;
    p->mass_scaling_k = 2.0f;
    p->wind_drag = 10.0f;
    p->wind_lift = 100.0f;
    p->rotation_iterations = 20;
    p->neighbor_skin = 0.0f;  // Verlet lists measured slower than the lambda-recorded lists (opt-in)
    // staging each CTA's neighbourhood in shared memory measured slower than
    // reading it through a full-size L1, and the contact walks' cell culling
    // pays only where solids dominate (both opt-in; bp_solver_autotune times them)
    p->walk_options = BP_WALK_NO_STAGING | BP_WALK_NO_CONTACT_CULLING;
    p->bending_stiffness = 0.8f;                   // bending.cuh:71
}

static bp_status check_params(const bp_params *p)
{
    if (!p) return fail(BP_ERR_INVALID_ARGUMENT, "params is NULL");
    if (p->mode != BP_MODE_REFERENCE && p->mode != BP_MODE_TEXTBOOK) return fail(BP_ERR_INVALID_ARGUMENT, "unknown mode");
    if (!is_pow2(p->grid_dim) || p->grid_dim < 4 || p->grid_dim > 512)
        return fail(BP_ERR_INVALID_ARGUMENT, "grid_dim must be a power of two in [4, 512]");
    if (!(p->cell_size > 0.f) || !(p->kernel_radius > 0.f) || !(p->rest_density > 0.f))
        return fail(BP_ERR_INVALID_ARGUMENT, "cell_size, kernel_radius and rest_density must be positive");
    if (p->kernel_radius > p->cell_size * 1.0001f)
        return fail(BP_ERR_INVALID_ARGUMENT, "kernel_radius must not exceed cell_size (27-cell search)");
    if (p->rotation_iterations < 0) return fail(BP_ERR_INVALID_ARGUMENT, "rotation_iterations < 0");
    if (!std::isfinite(p->bending_stiffness)) return fail(BP_ERR_INVALID_ARGUMENT, "bending_stiffness is not finite");
    if (p->scorr_n < 0 || p->scorr_n > 16) return fail(BP_ERR_INVALID_ARGUMENT, "scorr_n must be in [0, 16]");
    if (!(p->neighbor_skin >= 0.f)) return fail(BP_ERR_INVALID_ARGUMENT, "neighbor_skin < 0");
    if (p->scan_block != 0 && p->scan_block != 64 && p->scan_block != 128 && p->scan_block != 256)
        return fail(BP_ERR_INVALID_ARGUMENT, "scan_block must be 0, 64, 128 or 256");
    if (p->scan_persistent != 0 && p->scan_persistent != 1)
        return fail(BP_ERR_INVALID_ARGUMENT, "scan_persistent must be 0 or 1");
    return BP_OK;
}

// How far a particle may move from its hash-time position while walks skip
// the other alias classes of a table cell, or 0 when they may not skip them
// (see SimConsts::cls_perm).  A skipped particle was hashed in a real cell at
// least D cells from the walked one along some axis, so at least (D - 2)
// cells from the walker's cell; the hash's float rounding moves each cell
// boundary by less than 0.01 for |p| < 4e4 (checked by k_class_refresh), and
// 1e-3 h keeps the distance test's own rounding clear.  Taped updates walk
// whole cells (the adjoint re-runs do not record the classes).
// Whether the scene's planes hold it inside one period of the table on every
// axis: an axis-aligned box at most D - 2 cells wide, so that no 27-cell walk
// of a particle inside it meets two real cells in one table cell.  Such a
// scene gets no alias classes (their walks would skip nothing; a particle
// that leaves the box is still walked exactly, through whole table cells).
static bool planes_confine(const bp_solver *s, int D, float cell)
{
    for (int a = 0; a < 3; ++a) {
        float lo = -INFINITY, hi = INFINITY;
        for (int k = 0; k < s->nplanes; ++k) {
            const float *pl = s->planes[k];  // origin xyz, normal xyz
            const float n = pl[3 + a];
            if (!(fabsf(n) == 1.f && pl[3 + (a + 1) % 3] == 0.f && pl[3 + (a + 2) % 3] == 0.f)) continue;
            if (n > 0.f) lo = fmaxf(lo, pl[a]);
            else hi = fminf(hi, pl[a]);
        }
        if (!(hi - lo <= (float)(D - 2) * cell)) return false;
    }
    return true;
}

static float class_reach(const bp_solver *s)
{
    const bp_params &p = s->prm;
    if (!s->cls.perm || s->tape || (p.walk_options & BP_WALK_NO_ALIAS_CLASSES)) return 0.f;
    const float reach = (float)(s->cls_dmin - 2) * p.cell_size - p.kernel_radius - (0.02f + 1e-3f * p.kernel_radius);
    return reach > 0.f ? reach : 0.f;
}

// Substep constants: SetKernelRadius (K/fluid.cuh:11-27) evaluated on the host.
SimConsts bp::make_consts(const bp_solver *s, float sdt)
{
    const bp_params &p = s->prm;
    SimConsts C;
    memset(&C, 0, sizeof(C));
    C.n = s->n;
    C.D = p.grid_dim;
    C.mask = (unsigned)p.grid_dim - 1u;
    C.cell = p.cell_size;
    const float h = p.kernel_radius;
    C.h = h;
    C.h2 = h * h;
    C.half_h = h * 0.5f;
    C.c_poly6 = 315.f / 64.f / 3.141592f / powf(h, 9.0f);
    C.c_spiky = -45.f / 3.141592f / powf(h, 6.f);
    C.c_akinci = 32.0f / 3.141592f / powf(h, 9.f);
    C.c_akinci_off = powf(h, 6.0f) / 64.0f;
    if (p.mode == BP_MODE_TEXTBOOK) C.c_akinci_off = C.c_akinci * C.c_akinci_off;  // Akinci 2013 spline
    C.rho0 = p.rest_density;
    C.inv_rho0 = 1.0f / p.rest_density;
    C.solid_scale = p.solid_density_scale;
    C.lambda_den = p.lambda_denominator;
    C.relaxation = p.relaxation;
    C.textbook = p.mode == BP_MODE_TEXTBOOK;
    const bool akinci = (p.stage_mask & BP_STAGE_AKINCI) != 0;
    C.scorr_on = C.textbook || !akinci;
    C.clamp_c = akinci;
    C.scorr_k = p.scorr_k;
    C.scorr_ni = p.scorr_n;
    {
        const float dq = powf(p.scorr_dq * h, 2.f);
        const float t = C.h2 - dq;
        C.scorr_inv_wq = 1.0f / (C.c_poly6 * t * t * t);
    }
    C.delta_clamp = C.textbook ? -1.f : p.delta_clamp;  // textbook PBF has no per-pair clamp
    C.delta_clamp2 = C.delta_clamp * C.delta_clamp;
    C.vort_eps = p.vorticity_eps;
    C.tension = p.surface_tension;
    C.xsph_c = p.xsph_c;
    C.use_vort = (p.stage_mask & BP_STAGE_VORTICITY) != 0;
    C.use_akinci = akinci;
    C.use_xsph = (p.stage_mask & BP_STAGE_XSPH) != 0;
    C.radius = p.particle_radius;
    C.fs = p.friction_static;
    C.fd = p.friction_dynamic;
    C.mass_k = p.mass_scaling_k;
    C.gravity = make_float3(p.gravity[0], p.gravity[1], p.gravity[2]);
    C.wind = make_float3(p.wind_velocity[0], p.wind_velocity[1], p.wind_velocity[2]);
    C.wind_drag = p.wind_drag;
    C.wind_lift = p.wind_lift;
    C.rot_iters = p.rotation_iterations;
    C.dt = sdt;
    C.inv_dt = 1.0f / sdt;
    C.cell_keys = s->sorted_keys;  // stored cell of every particle (staged walks, Verlet lists)
    C.scn = s->scn;
    C.scene_of = s->scene_of;
    C.stage = (p.walk_options & BP_WALK_NO_STAGING) ? 0 : 1;
    C.split = (p.walk_options & BP_WALK_NO_SPLIT) ? 0 : 1;
    C.scan_block = p.scan_block > 0 ? p.scan_block : 256;
    C.scan_persist = p.scan_persistent ? 1 : 0;
    if (p.neighbor_skin > 0.f && !s->tape && s->vl) {  // Verlet lists (enqueue_substep decides per launch)
        C.vl = s->vl;
        C.vl_count = s->vl_count;
        C.vl_cap = kVerletCap;
        C.nl_cell = s->nl_cell;
        C.nl_pos = s->nl_pos;
        C.nl_outlier = s->nl_outlier;
        C.nl_zwords = (p.grid_dim + 63) / 64;
        const float hs = h * (1.0f + p.neighbor_skin);
        const float half_skin = 0.5f * h * p.neighbor_skin;
        C.nl_hs2 = hs * hs;
        C.nl_half_skin2 = half_skin * half_skin;
    }
    if (class_reach(s) > 0.f) {
        C.cls_perm = s->cls.perm;
        C.cls_inv = s->cls.inv;
        C.cls_of = s->cls.cls;
        C.cls_off = s->cls.off;
        C.cls_pos = s->cls.pos;
        C.cls_moved = s->cls.moved;
        C.cls_T = s->cls.T;
        C.cls_mass = s->cls.mass;
        C.cls_lm = s->cls.lm;
        C.cls_rho = s->cls.rho;
        C.cls_vel = s->cls.vel;
        C.cls_om = s->cls.om;
        C.cls_nm = s->cls.nm;
        C.cls_vb = s->cls.vb;
    }
    C.nplanes = (p.stage_mask & BP_STAGE_PLANES) ? s->nplanes : 0;
    for (int k = 0; k < s->nplanes; ++k) {
        C.plane_o[k] = make_float4(s->planes[k][0], s->planes[k][1], s->planes[k][2], 0.f);
        C.plane_n[k] = make_float4(s->planes[k][3], s->planes[k][4], s->planes[k][5], 0.f);
    }
    return C;
}

// Builds CSR incidence lists (node = original particle id) for a set of
// constraints that each touch `arity` particles.
static void build_incidence(int n, int count, int arity, const int32_t *ids, bool encode_side,
                            std::vector<int> &nodes, std::vector<int> &ptr, std::vector<int> &inc)
{
    std::vector<int> deg(n, 0);
    for (int c = 0; c < count; ++c)
        for (int a = 0; a < arity; ++a) deg[ids[arity * c + a]]++;
    std::vector<int> node_of(n, -1);
    nodes.clear();
    for (int i = 0; i < n; ++i)
        if (deg[i]) {
            node_of[i] = (int)nodes.size();
            nodes.push_back(i);
        }
    ptr.assign(nodes.size() + 1, 0);
    for (size_t k = 0; k < nodes.size(); ++k) ptr[k + 1] = ptr[k] + deg[nodes[k]];
    inc.assign(ptr.back(), 0);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int c = 0; c < count; ++c)
        for (int a = 0; a < arity; ++a) {
            const int nd = node_of[ids[arity * c + a]];
            inc[fill[nd]++] = encode_side ? (c * arity + a) : c;
        }
}

static bp_status validate_scene(const bp_scene_desc *sc)
{
    if (!sc) return fail(BP_ERR_INVALID_ARGUMENT, "scene is NULL");
    const int n = sc->num_particles;
    if (n < 0) return fail(BP_ERR_INVALID_ARGUMENT, "num_particles < 0");
    if (n > (1 << 28)) return fail(BP_ERR_CAPACITY, "num_particles above 2^28");
    if (n > 0 && (!sc->positions || !sc->masses || !sc->phases))
        return fail(BP_ERR_INVALID_ARGUMENT, "positions, masses and phases are required");
    for (int i = 0; i < n; ++i) {
        if (sc->phases[i] == 0) return fail(BP_ERR_INVALID_ARGUMENT, "phase 0 is reserved (fluid < 0, solid > 0)");
        if (!(sc->masses[i] > 0.f)) return fail(BP_ERR_INVALID_ARGUMENT, "masses must be positive");
    }
    if (sc->num_planes < 0 || sc->num_planes > kMaxPlanes)
        return fail(BP_ERR_CAPACITY, "at most 16 planes");
    if (sc->num_planes > 0 && !sc->planes) return fail(BP_ERR_INVALID_ARGUMENT, "planes is NULL");
    auto check_ids = [&](int count, int arity, const int32_t *ids, const char *what) -> bp_status {
        if (count < 0) return fail(BP_ERR_INVALID_ARGUMENT, std::string(what) + ": negative count");
        if (count > 0 && !ids) return fail(BP_ERR_INVALID_ARGUMENT, std::string(what) + ": NULL");
        for (long k = 0; k < (long)count * arity; ++k)
            if (ids[k] < 0 || ids[k] >= n) return fail(BP_ERR_INVALID_ARGUMENT, std::string(what) + ": id out of range");
        return BP_OK;
    };
    bp_status st;
    if ((st = check_ids(sc->num_distance_constraints, 2, sc->distance_pairs, "distance_pairs")) != BP_OK) return st;
    if (sc->num_distance_constraints > 0 && !sc->distance_params)
        return fail(BP_ERR_INVALID_ARGUMENT, "distance_params is NULL");
    if ((st = check_ids(sc->num_wind_faces, 3, sc->wind_faces, "wind_faces")) != BP_OK) return st;
    if ((st = check_ids(sc->num_immovables, 1, sc->immovables, "immovables")) != BP_OK) return st;
    if ((st = check_ids(sc->num_bendings, 4, sc->bendings, "bendings")) != BP_OK) return st;
    if (sc->num_rigid_bodies < 0) return fail(BP_ERR_INVALID_ARGUMENT, "num_rigid_bodies < 0");
    if (sc->num_rigid_bodies > 0 && (!sc->rigid_ranges || !sc->rigid_rest_positions))
        return fail(BP_ERR_INVALID_ARGUMENT, "rigid_ranges / rigid_rest_positions is NULL");
    for (int b = 0; b < sc->num_rigid_bodies; ++b) {
        const int r0 = sc->rigid_ranges[2 * b], r1 = sc->rigid_ranges[2 * b + 1];
        if (r0 < 0 || r1 > n || r1 <= r0) return fail(BP_ERR_INVALID_ARGUMENT, "rigid range out of bounds");
    }
    return BP_OK;
}

// The scenes of a batched ensemble: per-scene grids and constants.
struct BatchSpec {
    std::vector<int> first;             // particle offsets, num_scenes + 1
    std::vector<SceneConsts> scenes;
    size_t ncells = 0;
    int sort_dim = 0;
    int max_planes = 0;
};

static bp_status create_solver(const bp_scene_desc *sc, const bp_params *prm, void *stream, const BatchSpec *batch,
                               bp_solver **out)
{
    if (!out) return fail(BP_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    bp_status st;
    if ((st = validate_scene(sc)) != BP_OK) return st;
    if ((st = check_params(prm)) != BP_OK) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(BP_ERR_NO_DEVICE, "no CUDA device visible");
    }
    bp_solver *s = new (std::nothrow) bp_solver();
    if (!s) return fail(BP_ERR_OUT_OF_MEMORY, "host allocation failed");
    auto bail = [&](bp_status e) {
        delete s;
        return e;
    };
    const int n = sc->num_particles;
    s->n = n;
    s->prm = *prm;
    s->nplanes = sc->num_planes;
    for (int k = 0; k < s->nplanes; ++k)
        for (int c = 0; c < 6; ++c) s->planes[k][c] = sc->planes[6 * k + c];
    cudaGetDevice(&s->device);
    if (stream) {
        s->stream = (cudaStream_t)stream;
    } else {
        // graphs cannot be captured on the legacy stream; a blocking stream
        // still orders itself with it, like the reference's default-stream use
        if (cudaStreamCreate(&s->stream) != cudaSuccess) return bail(fail(BP_ERR_CUDA, "cudaStreamCreate failed"));
        s->own_stream = true;
    }

    const size_t N = (size_t)(n > 0 ? n : 1);
    const int D = prm->grid_dim;
    const size_t ncells = batch ? batch->ncells : (size_t)D * D * D;
    s->ncells = ncells;
    s->sort_dim = batch ? batch->sort_dim : D;
    const size_t NM = batch ? 1 : N;  // Verlet lists: single scenes only
    if ((st = s->alloc(&s->Xc, N)) || (st = s->alloc(&s->Vc, N)) || (st = s->alloc(&s->Xs, N)) ||
        (st = s->alloc(&s->Vs, N)) || (st = s->alloc(&s->Pa, N)) || (st = s->alloc(&s->Pb, N)) ||
        (st = s->alloc(&s->Om, N)) || (st = s->alloc(&s->Nm, N)) || (st = s->alloc(&s->orig_c, N)) ||
        (st = s->alloc(&s->orig_s, N)) || (st = s->alloc(&s->to_new, N)) || (st = s->alloc(&s->group, N)) ||
        (st = s->alloc(&s->keys, N)) || (st = s->alloc(&s->sorted_keys, N)) || (st = s->alloc(&s->order, N)) ||
        (st = s->alloc(&s->off, ncells + 1)) || (st = s->alloc(&s->mass, N)) || (st = s->alloc(&s->lam, N)) || (st = s->alloc(&s->lm, N)) ||
        (st = s->alloc(&s->rho, N)) || (st = s->alloc(&s->w, N)) || (st = s->alloc(&s->err, 1)) ||
        (st = s->alloc(&s->staging, 6 * N)) || (st = s->alloc(&s->vl, NM * kVerletCap)) ||
        (st = s->alloc(&s->nl_cell, NM)) || (st = s->alloc(&s->nl_pos, NM)) ||
        (st = s->alloc(&s->nl_outlier, (size_t)D * D * ((D + 63) / 64))) ||
        (st = s->alloc(&s->vl_count, NM)) || (st = s->alloc(&s->nl_stats, 5)))
        return bail(st);
    {
        char *scratch = nullptr;
        if ((st = s->alloc(&scratch, sort_scratch_bytes((int)N, s->sort_dim)))) return bail(st);
        sort_scratch_carve(scratch, (int)N, s->sort_dim, &s->sort);
    }
    if (ncells <= kClassMaxCells && (batch || !planes_confine(s, D, prm->cell_size))) {
        ClassArrays &a = s->cls;
        if ((st = s->alloc(&a.cls, N)) || (st = s->alloc(&a.pos0, N)) || (st = s->alloc(&a.keys, N)) ||
            (st = s->alloc(&a.perm, N)) || (st = s->alloc(&a.inv, N)) || (st = s->alloc(&a.off, 8 * ncells + 1)) ||
            (st = s->alloc(&a.pos, N)) || (st = s->alloc(&a.mixed, 1)) || (st = s->alloc(&a.moved, 1)) ||
            (st = s->alloc(&a.mass, N)) || (st = s->alloc(&a.lm, N)) || (st = s->alloc(&a.rho, N)) ||
            (st = s->alloc(&a.vel, N)) || (st = s->alloc(&a.om, N)) || (st = s->alloc(&a.nm, N)) ||
            (st = s->alloc(&a.vb, N)))
            return bail(st);
        a.T = (int)ncells;
        s->cls_dmin = D;
        if (batch)
            for (const SceneConsts &c : batch->scenes) s->cls_dmin = std::min(s->cls_dmin, c.D);
    }

    // initial state in original order (sorted order == identity)
    std::vector<float4> X(N), V(N), P(N);
    std::vector<int> ids(N), grp(N, 0);
    bool has_solid = false;
    for (int i = 0; i < n; ++i) {
        const float *x = sc->positions + 3 * i;
        const float *v = sc->velocities ? sc->velocities + 3 * i : nullptr;
        int ph = sc->phases[i];
        has_solid |= ph > 0;
        float phf;
        memcpy(&phf, &ph, 4);
        X[i] = make_float4(x[0], x[1], x[2], sc->masses[i]);
        V[i] = make_float4(v ? v[0] : 0.f, v ? v[1] : 0.f, v ? v[2] : 0.f, phf);
        P[i] = make_float4(x[0], x[1], x[2], phf);
        ids[i] = i;
        if (sc->group_ids) grp[i] = sc->group_ids[i];
    }
    s->has_solid = has_solid;
    s->num_solids = 0;
    for (int i = 0; i < n; ++i) s->num_solids += sc->phases[i] > 0;
    if ((st = s->alloc(&s->tile_solid, (N + 255) / 256)) || (st = s->alloc(&s->solid_prefix, N + 1)) ||
        (st = s->alloc(&s->solid_pos, N + 1)) ||  // phases may change after creation: room for every particle
        (st = s->alloc(&s->solid_list, N)) || (st = s->alloc(&s->solid_totals, (N + 1023) / 1024)) ||
        (st = s->alloc(&s->nbr, N * kPostListCap)) ||
        (st = s->alloc(&s->walk_xyz, 4 * (((N + 3) & ~(size_t)3) + kPlanePad))) ||
        (st = s->alloc(&s->nbr_count, N)))
        return bail(st);
    s->walk_stride = (int)(((N + 3) & ~(size_t)3) + kPlanePad);
    BP_CUDA_BAIL(cudaMemset(s->walk_xyz, 0, 4 * (size_t)s->walk_stride * sizeof(float)));
    // contact walks restricted to the cells a partner can be stored in
    if (has_solid && ((st = s->alloc(&s->hash_pos, N)) || (st = s->alloc(&s->contact_reach, 2)) ||
                      (st = s->alloc(&s->solid_walk, N))))
        return bail(st);
    // fluid next to solids: the cell masks that let fluid far from every
    // solid skip its walk over the solids (one scene's table)
    if (!batch && s->num_solids > 0 && s->num_solids < n &&
        ((st = s->alloc(&s->solid_cells, ncells / 64)) || (st = s->alloc(&s->solid_near, ncells / 64))))
        return bail(st);
    if (n > 0) {
        BP_CUDA_BAIL(cudaMemcpy(s->Xc, X.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
        BP_CUDA_BAIL(cudaMemcpy(s->Vc, V.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
        BP_CUDA_BAIL(cudaMemcpy(s->Pa, P.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
        BP_CUDA_BAIL(cudaMemcpy(s->orig_c, ids.data(), n * sizeof(int), cudaMemcpyHostToDevice));
        BP_CUDA_BAIL(cudaMemcpy(s->to_new, ids.data(), n * sizeof(int), cudaMemcpyHostToDevice));
        BP_CUDA_BAIL(cudaMemcpy(s->group, grp.data(), n * sizeof(int), cudaMemcpyHostToDevice));
        std::vector<float> m(sc->masses, sc->masses + n);
        BP_CUDA_BAIL(cudaMemcpy(s->mass, m.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    }
    s->Pcur = s->Pa;
    BP_CUDA_BAIL(cudaMemset(s->lam, 0, N * sizeof(float)));
    BP_CUDA_BAIL(cudaMemset(s->rho, 0, N * sizeof(float)));
    BP_CUDA_BAIL(cudaMemset(s->Om, 0, N * sizeof(float4)));
    BP_CUDA_BAIL(cudaMemset(s->Nm, 0, N * sizeof(float4)));
    BP_CUDA_BAIL(cudaMemset(s->off, 0, (ncells + 1) * sizeof(int)));
    BP_CUDA_BAIL(cudaMemset(s->sorted_keys, 0, N * sizeof(int)));
    BP_CUDA_BAIL(cudaMemset(s->err, 0, sizeof(unsigned)));

    // distance constraints
    if (sc->num_distance_constraints > 0) {
        const int m = sc->num_distance_constraints;
        std::vector<int> nodes, ptr, inc;
        build_incidence(n, m, 2, sc->distance_pairs, true, nodes, ptr, inc);
        s->dist.num_edges = m;
        s->dist.num_nodes = (int)nodes.size();
        int2 *pairs;
        float2 *params;
        int *nid, *nptr, *ninc;
        float4 *ek;
        if ((st = s->upload(&pairs, sc->distance_pairs, m)) || (st = s->upload(&params, sc->distance_params, m)) ||
            (st = s->upload(&nid, nodes.data(), nodes.size())) || (st = s->upload(&nptr, ptr.data(), ptr.size())) ||
            (st = s->upload(&ninc, inc.data(), inc.size())) || (st = s->alloc(&ek, m)))
            return bail(st);
        s->dist.pairs = pairs;
        s->dist.params = params;
        s->dist.node_ids = nid;
        s->dist.node_ptr = nptr;
        s->dist.node_inc = ninc;
        s->dist.edge_k = ek;
    }
    if (sc->num_bendings > 0) {
        const int q = sc->num_bendings;
        std::vector<int> nodes, ptr, inc;
        build_incidence(n, q, 4, sc->bendings, true, nodes, ptr, inc);
        s->bend.num_quads = q;
        s->bend.num_nodes = (int)nodes.size();
        int4 *quads;
        int *nid, *nptr, *ninc;
        float4 *terms;
        if ((st = s->upload(&quads, sc->bendings, q)) || (st = s->upload(&nid, nodes.data(), nodes.size())) ||
            (st = s->upload(&nptr, ptr.data(), ptr.size())) || (st = s->upload(&ninc, inc.data(), inc.size())) ||
            (st = s->alloc(&terms, 4 * (size_t)q)))
            return bail(st);
        s->bend.quads = quads;
        s->bend.node_ids = nid;
        s->bend.node_ptr = nptr;
        s->bend.node_inc = ninc;
        s->bend.terms = terms;
    }
    if (sc->num_wind_faces > 0) {
        const int f = sc->num_wind_faces;
        std::vector<int> nodes, ptr, inc;
        build_incidence(n, f, 3, sc->wind_faces, false, nodes, ptr, inc);
        s->wind.num_faces = f;
        s->wind.num_nodes = (int)nodes.size();
        int *faces, *nid, *nptr, *ninc;
        float4 *mv;
        if ((st = s->upload(&faces, sc->wind_faces, 3 * (size_t)f)) || (st = s->upload(&nid, nodes.data(), nodes.size())) ||
            (st = s->upload(&nptr, ptr.data(), ptr.size())) || (st = s->upload(&ninc, inc.data(), inc.size())) ||
            (st = s->alloc(&mv, f)))
            return bail(st);
        s->wind.faces = faces;
        s->wind.node_ids = nid;
        s->wind.node_ptr = nptr;
        s->wind.node_inc = ninc;
        s->wind.face_move = mv;
    }
    if (sc->num_rigid_bodies > 0) {
        const int b = sc->num_rigid_bodies;
        std::vector<float4> rest(N, make_float4(0.f, 0.f, 0.f, 0.f));
        for (int i = 0; i < n; ++i)
            rest[i] = make_float4(sc->rigid_rest_positions[3 * i], sc->rigid_rest_positions[3 * i + 1],
                                  sc->rigid_rest_positions[3 * i + 2], 0.f);
        std::vector<float4> rot(b, make_float4(0.f, 0.f, 0.f, 1.f)), cm(b, make_float4(0.f, 0.f, 0.f, 0.f));
        int2 *ranges;
        float4 *drest, *drot, *dcm;
        if ((st = s->upload(&ranges, sc->rigid_ranges, b)) || (st = s->upload(&drest, rest.data(), N)) ||
            (st = s->upload(&drot, rot.data(), b)) || (st = s->upload(&dcm, cm.data(), b)))
            return bail(st);
        s->rigid.num_bodies = b;
        s->rigid.ranges = ranges;
        s->rigid.rest = drest;
        s->rigid.rot = drot;
        s->rigid.cm = dcm;
    }
    if (sc->num_immovables > 0) {
        s->nimm = sc->num_immovables;
        if ((st = s->upload(&s->imm, sc->immovables, s->nimm))) return bail(st);
    }
    if (batch) {
        const int S = (int)batch->scenes.size();
        std::vector<int> of(N, 0);
        for (int k = 0; k < S; ++k)
            for (int i = batch->first[k]; i < batch->first[k + 1]; ++i) of[i] = k;
        if ((st = s->upload(&s->scn, batch->scenes.data(), S)) || (st = s->upload(&s->scene_of, of.data(), N)))
            return bail(st);
        s->num_scenes = S;
        s->scene_first = batch->first;
        s->nplanes = batch->max_planes;  // each scene's own planes are in its table entry
    }
    BP_CUDA_BAIL(cudaDeviceSynchronize());
    *out = s;
    return BP_OK;
}

extern "C" bp_status bp_solver_create(const bp_scene_desc *sc, const bp_params *prm, void *stream, bp_solver **out)
{
    return create_solver(sc, prm, stream, nullptr, out);
}

// Parameters that scenes of one batch may not differ in: everything except
// rest density, gravity and grid dimension.
static bool same_shared_params(const bp_params &a, const bp_params &b)
{
    bp_params x = a, y = b;
    for (bp_params *p : {&x, &y}) {
        p->rest_density = 0.f;
        p->gravity[0] = p->gravity[1] = p->gravity[2] = 0.f;
        p->grid_dim = 0;
    }
    return memcmp(&x, &y, sizeof(bp_params)) == 0;
}

extern "C" bp_status bp_batch_create(int32_t num_scenes, const bp_scene_desc *scenes, const bp_params *params,
                                     void *stream, bp_solver **out)
{
    if (!out) return fail(BP_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (num_scenes <= 0 || !scenes || !params) return fail(BP_ERR_INVALID_ARGUMENT, "no scenes");
    bp_status st;
    BatchSpec spec;
    spec.first.assign(num_scenes + 1, 0);
    spec.scenes.resize(num_scenes);
    int64_t total = 0;
    size_t cells = 0;
    for (int k = 0; k < num_scenes; ++k) {
        if ((st = validate_scene(&scenes[k])) != BP_OK) return st;
        if ((st = check_params(&params[k])) != BP_OK) return st;
        if (!same_shared_params(params[0], params[k]))
            return fail(BP_ERR_INVALID_ARGUMENT,
                        "scenes of a batch differ only in rest_density, gravity and grid_dim");
        if (params[k].neighbor_skin > 0.f)
            return fail(BP_ERR_INVALID_ARGUMENT, "Verlet lists (neighbor_skin > 0) are not available in a batch");
        spec.first[k] = (int)total;
        total += scenes[k].num_particles;
        if (total > (1 << 28)) return fail(BP_ERR_CAPACITY, "a batch holds at most 2^28 particles");
        SceneConsts &c = spec.scenes[k];
        memset(&c, 0, sizeof(c));
        const int D = params[k].grid_dim;
        c.D = D;
        c.mask = (unsigned)D - 1u;
        c.base = (int)cells;
        cells += (size_t)D * D * D;
        if (cells >= ((size_t)1 << 30)) return fail(BP_ERR_CAPACITY, "a batch's grids hold at most 2^30 cells");
        c.rho0 = params[k].rest_density;
        c.inv_rho0 = 1.0f / params[k].rest_density;
        c.gx = params[k].gravity[0];
        c.gy = params[k].gravity[1];
        c.gz = params[k].gravity[2];
        c.nplanes = scenes[k].num_planes;
        for (int q = 0; q < c.nplanes; ++q) {
            const float *pl = scenes[k].planes + 6 * q;
            c.plane_o[q] = make_float4(pl[0], pl[1], pl[2], 0.f);
            c.plane_n[q] = make_float4(pl[3], pl[4], pl[5], 0.f);
        }
        spec.max_planes = std::max(spec.max_planes, c.nplanes);
    }
    spec.first[num_scenes] = (int)total;
    spec.ncells = cells;
    spec.sort_dim = 4;
    while ((size_t)spec.sort_dim * spec.sort_dim * spec.sort_dim < cells) spec.sort_dim *= 2;

    // one scene description: the scenes' particles and constraints concatenated, ids offset
    const int n = (int)total;
    std::vector<float> pos(3 * (size_t)n), vel(3 * (size_t)n, 0.f), mass(n), rest;
    std::vector<int32_t> phase(n), group(n, 0), pairs, faces, ranges, imm, quads;
    std::vector<float> dparams;
    bool any_rigid = false;
    for (int k = 0; k < num_scenes; ++k) any_rigid |= scenes[k].num_rigid_bodies > 0;
    if (any_rigid) rest.assign(3 * (size_t)n, 0.f);
    for (int k = 0; k < num_scenes; ++k) {
        const bp_scene_desc &d = scenes[k];
        const int o = spec.first[k], m = d.num_particles;
        if (m == 0) continue;
        std::copy(d.positions, d.positions + 3 * (size_t)m, pos.begin() + 3 * (size_t)o);
        if (d.velocities) std::copy(d.velocities, d.velocities + 3 * (size_t)m, vel.begin() + 3 * (size_t)o);
        std::copy(d.masses, d.masses + m, mass.begin() + o);
        std::copy(d.phases, d.phases + m, phase.begin() + o);
        if (d.group_ids) std::copy(d.group_ids, d.group_ids + m, group.begin() + o);
        for (int e = 0; e < 2 * d.num_distance_constraints; ++e) pairs.push_back(d.distance_pairs[e] + o);
        dparams.insert(dparams.end(), d.distance_params, d.distance_params + 2 * (size_t)d.num_distance_constraints);
        for (int e = 0; e < 3 * d.num_wind_faces; ++e) faces.push_back(d.wind_faces[e] + o);
        for (int e = 0; e < 2 * d.num_rigid_bodies; ++e) ranges.push_back(d.rigid_ranges[e] + o);
        if (d.num_rigid_bodies > 0)
            std::copy(d.rigid_rest_positions, d.rigid_rest_positions + 3 * (size_t)m, rest.begin() + 3 * (size_t)o);
        for (int e = 0; e < d.num_immovables; ++e) imm.push_back(d.immovables[e] + o);
        for (int e = 0; e < 4 * d.num_bendings; ++e) quads.push_back(d.bendings[e] + o);
    }
    bp_scene_desc all;
    memset(&all, 0, sizeof(all));
    all.num_particles = n;
    all.positions = pos.data();
    all.velocities = vel.data();
    all.masses = mass.data();
    all.phases = phase.data();
    all.group_ids = group.data();
    all.num_distance_constraints = (int)(pairs.size() / 2);
    all.distance_pairs = pairs.data();
    all.distance_params = dparams.data();
    all.num_wind_faces = (int)(faces.size() / 3);
    all.wind_faces = faces.data();
    all.num_rigid_bodies = (int)(ranges.size() / 2);
    all.rigid_ranges = ranges.data();
    all.rigid_rest_positions = any_rigid ? rest.data() : nullptr;
    all.num_immovables = (int)imm.size();
    all.immovables = imm.data();
    all.num_bendings = (int)(quads.size() / 4);
    all.bendings = quads.data();
    bp_params shared = params[0];
    shared.grid_dim = 4;  // unused: every particle walks its scene's grid
    return create_solver(&all, &shared, stream, &spec, out);
}

extern "C" bp_status bp_batch_step(bp_solver *s, float dt, int32_t num_substeps, int32_t iterations)
{
    if (s && s->num_scenes == 0) return fail(BP_ERR_INVALID_ARGUMENT, "not a batch (use bp_solver_step)");
    return bp_solver_step(s, dt, num_substeps, iterations);
}

extern "C" bp_status bp_batch_scene_range(const bp_solver *s, int32_t scene, int32_t *first, int32_t *count)
{
    if (!s || !first || !count) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (s->num_scenes == 0) return fail(BP_ERR_INVALID_ARGUMENT, "not a batch");
    if (scene < 0 || scene >= s->num_scenes) return fail(BP_ERR_INVALID_ARGUMENT, "scene out of range");
    *first = s->scene_first[scene];
    *count = s->scene_first[scene + 1] - s->scene_first[scene];
    return BP_OK;
}

extern "C" bp_status bp_solver_destroy(bp_solver *s)
{
    if (!s) return BP_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    delete s;
    return BP_OK;
}

extern "C" bp_status bp_solver_get_params(const bp_solver *s, bp_params *out)
{
    if (!s || !out) return fail(BP_ERR_INVALID_ARGUMENT, "solver or output is NULL");
    *out = s->prm;
    return BP_OK;
}

extern "C" bp_status bp_solver_set_params(bp_solver *s, const bp_params *prm)
{
    if (!s) return fail(BP_ERR_INVALID_ARGUMENT, "solver is NULL");
    bp_status st = check_params(prm);
    if (st != BP_OK) return st;
    if (s->num_scenes > 0) {
        // a batch keeps each scene's grid, rest density and gravity from creation
        if (prm->neighbor_skin > 0.f)
            return fail(BP_ERR_INVALID_ARGUMENT, "Verlet lists (neighbor_skin > 0) are not available in a batch");
        const int D = s->prm.grid_dim;
        s->prm = *prm;
        s->prm.grid_dim = D;
    } else {
        if (prm->grid_dim != s->prm.grid_dim)
            return fail(BP_ERR_INVALID_ARGUMENT, "grid_dim cannot change after creation");
        s->prm = *prm;
    }
    s->params_version++;
    return BP_OK;
}

// Enqueues one substep; returns the number of kernels launched.
void bp::enqueue_substep(bp_solver *s, const SimConsts &C, int iterations, int picked, float3 ppos, LaunchLog *L,
                         SubstepTape *tape)
{
    const cudaStream_t st = s->stream;
    const int mask = s->prm.stage_mask;
    const bool planes = (mask & BP_STAGE_PLANES) && s->nplanes > 0;
    const bool wind = (mask & BP_STAGE_WIND) && s->wind.num_faces > 0;
    const bool pcoll = (mask & BP_STAGE_PARTICLE_COLLISION) && s->has_solid;
    const bool fluid = (mask & BP_STAGE_FLUID) != 0;
    const bool distance = (mask & BP_STAGE_DISTANCE) && s->dist.num_edges > 0;
    const bool bending = (mask & BP_STAGE_BENDING) && s->bend.num_quads > 0;
    const bool rigid = (mask & BP_STAGE_SHAPE_MATCHING) && s->rigid.num_bodies > 0;
    const bool immov = (mask & BP_STAGE_IMMOVABLE) && s->nimm > 0;
    const bool picking = picked >= 0;
    const bool tail = distance || bending || rigid || immov;  // stages after the fluid position pass
    if (picking) launch_pick(st, picked, s->to_new, s->Xc, ppos, 1, s->Vc, make_float3(0.f, 0.f, 0.f), L);

    launch_hash_state(st, C, s->Xc, s->Vc, s->keys, s->sort.hist, L);
    radix_sort_pairs(st, s->n, s->sort_dim, s->keys, nullptr, s->sorted_keys, s->order, s->sort, true, L);
    launch_cell_offsets(st, s->n, (int)s->ncells, s->sorted_keys, s->off, L);

    // iteration fusion: the reorder takes iteration 0's plane collision, and the
    // position pass the next iteration's or the final commit (BP_WALK_NO_FUSION:
    // launches of their own; bit-identical either way)
    const bool fuse = !tape && !(s->prm.walk_options & BP_WALK_NO_FUSION);
    const bool fuse_first_planes = planes && !wind && !picking && iterations > 0 && fuse;
    ReorderArgs ra;
    ra.order = s->order;
    ra.Xc = s->Xc;
    ra.Vc = s->Vc;
    ra.orig_c = s->orig_c;
    ra.Xs = s->Xs;
    ra.Vs = s->Vs;
    ra.P = s->Pa;
    ra.mass = s->mass;
    ra.orig_s = s->orig_s;
    ra.to_new = s->to_new;
    ra.inv_scaled = (distance || bending || pcoll) ? s->w : nullptr;
    ra.stabilize = planes;
    ra.collide = fuse_first_planes;
    ra.tile_solid = pcoll ? s->tile_solid : nullptr;
    if (pcoll) cudaMemsetAsync(s->tile_solid, 0, ((s->n + 255) / 256) * sizeof(int), st);
    const bool classes = C.cls_perm != nullptr;
    ClassArrays ca = s->cls;
    {
        const float r = class_reach(s);
        ca.reach2 = r * r;
    }
    ra.cls = classes ? ca.cls : nullptr;
    ra.pos0 = classes ? ca.pos0 : nullptr;
    // the contact walks' reach (BP_WALK_NO_CONTACT_CULLING: the 27 cells)
    const bool culling = pcoll && s->hash_pos && !(s->prm.walk_options & BP_WALK_NO_CONTACT_CULLING);
    // the solids' own walks are culled (and their walkers grouped by octant)
    // only where solids are at least half the particles (launch_contact_reach)
    const bool solid_culling = culling && 2LL * s->num_solids >= s->n;
    ra.hash_pos = culling ? s->hash_pos : nullptr;
    launch_reorder(st, C, ra, L);
    if (classes) launch_class_order(st, s->n, s->sorted_keys, s->off, s->mass, ca, s->sort, L);
    // walks read candidates in class order: gather P before each walking launch
    auto refresh = [&](const float4 *P) {
        if (classes) launch_class_refresh(st, s->n, P, ca, L);
    };
    if (tape) tape->vs_slot = tape->snap4(s->Vs);

    float4 *cur = s->Pa, *other = s->Pb;
    // Verlet lists (SimConsts::vl): iteration 0's lambda builds them and every
    // later walk of the substep may read them; the kernels before the build
    // neither read them nor track displacements.
    const bool verlet = C.vl != nullptr && fluid && iterations > 0;
    SimConsts Cpre = C;
    Cpre.vl = nullptr;
    Cpre.nl_pos = nullptr;
    const SimConsts &Cpost = verlet ? C : Cpre;
    // Without them lambda records each particle's neighbours within h for the
    // position pass (the same positions), which then reads them instead of
    // walking cells.
    const bool lists = !(s->prm.walk_options & BP_WALK_NO_LISTS) && s->nbr;
    // With Verlet lists the later lambda passes read them and record the exact
    // lists as well; the pass that builds them does not, so the position pass
    // right after it reads the Verlet lists instead.
    // The recording walks of the lambda pass and post pass A read their
    // candidates from the walk planes, written just before them
    // (BP_WALK_NO_PLANES: from the position records).
    const bool walk_planes = lists && !verlet && s->walk_xyz && C.split && !C.stage &&
                        !(s->prm.walk_options & BP_WALK_NO_PLANES);
    auto refresh_planes = [&](const float4 *P) {
        if (classes) launch_class_refresh(st, s->n, P, ca, L, nullptr, s->walk_xyz, s->walk_stride);
        else launch_walk_planes(st, s->n, P, s->walk_xyz, s->walk_stride, L);
    };
    SimConsts Cf = Cpost;
    if (lists) {
        Cf.nbr = s->nbr;
        Cf.nbr_count = s->nbr_count;
        Cf.nbr_cap = kPostListCap;
        Cf.lm = s->lm;
    }
    if (walk_planes) {
        Cf.walk_xyz = s->walk_xyz;
        Cf.walk_stride = s->walk_stride;
    }
    SimConsts Cbuild = verlet ? Cpost : Cf;
    Cbuild.vl_build = verlet ? 1 : 0;

    // the sorted order is fixed for the substep: compact its solids once
    if (pcoll) {
        SolidCells sc;
        if (s->solid_cells) {
            sc.D = C.D;
            sc.keys = s->sorted_keys;
            sc.cells = s->solid_cells;
            sc.near = s->solid_near;
        }
        launch_solid_list(st, s->n, cur, s->solid_totals, s->solid_prefix, s->solid_list, sc, L, s->num_solids,
                          C.cell, solid_culling ? s->solid_walk : nullptr);
    }
    if (wind) {
        if (tape) tape->push(TS_WIND, cur);
        launch_wind(st, Cpre, s->wind, cur, s->Vs, s->mass, s->to_new, L);
    }

    bool planes_done = fuse_first_planes;
    bool committed = false;
    for (int it = 0; it < iterations; ++it) {
        const SimConsts &Cit = it == 0 ? Cpre : Cpost;  // stages before lambda
        if (picking) {
            if (tape) tape->mark(TS_PICK);
            launch_pick(st, picked, s->to_new, cur, ppos, 1, nullptr, make_float3(0.f, 0.f, 0.f), L);
        }
        if (planes && !planes_done) {
            if (tape) tape->push(TS_PLANES, cur);
            launch_planes(st, Cit, s->Xs, cur, L);
        }
        planes_done = false;
        if (pcoll) {
            if (tape) tape->push(TS_PCOLL, cur);
            // solids walk in a launch of their own, in full warps (measured
            // faster than walking them in the staged CTAs, whether solids are
            // scattered through fluid or the whole scene)
            refresh(cur);
            SimConsts Cc = Cit;
            if (culling) {
                launch_contact_reach(st, s->n, cur, s->hash_pos, s->contact_reach, L, s->num_solids,
                                     s->solid_prefix, s->solid_list);
                Cc.contact_reach = s->contact_reach;
            }
            launch_particle_collision(st, Cc, cur, s->Xs, s->w, s->off, s->tile_solid, s->solid_prefix,
                                      s->solid_list, solid_culling ? s->solid_walk : nullptr, s->num_solids, true,
                                      s->solid_near, s->solid_pos, other, L);
            std::swap(cur, other);
        }
        if (fluid) {
            // lambda and delta-p read the same positions
            if (walk_planes) refresh_planes(cur);
            else refresh(cur);
            if (verlet && it == 0)
                cudaMemsetAsync(s->nl_outlier, 0, (size_t)C.D * C.D * C.nl_zwords * sizeof(unsigned long long), st);
            launch_lambda(st, it == 0 ? Cbuild : Cf, cur, s->mass, s->off, s->lam, s->rho, L);
            if (tape) {
                const int aux = tape->snap1(s->lam);
                tape->snap1(s->rho);
                tape->push(TS_FLUID, cur, aux);
            }
            DeltaArgs da;
            da.P = cur;
            da.mass = s->mass;
            da.lam = s->lam;
            da.off = s->off;
            da.Pout = other;
            da.epilogue = 0;
            da.Xs = s->Xs;
            da.Xc = s->Xc;
            da.Vc = s->Vc;
            da.Vs = s->Vs;
            da.orig_s = s->orig_s;
            da.orig_c = s->orig_c;
            if (!tail && fuse) {
                if (it == iterations - 1) {
                    da.epilogue = 2;
                    committed = true;
                } else if (planes && !picking) {
                    da.epilogue = 1;
                    planes_done = true;
                }
            }
            launch_deltap(st, (verlet && it == 0) ? Cpost : Cf, da, L);
            std::swap(cur, other);
        }
        if (distance) {
            if (tape) tape->push(TS_DISTANCE, cur);
            launch_distance(st, Cpost, s->dist, cur, s->w, s->to_new, s->err, L);
        }
        if (bending) {  // PS:956-969
            if (tape) tape->push(TS_BENDING, cur);
            BendingArgs ba = s->bend;
            ba.stiffness = s->prm.bending_stiffness;
            launch_bending(st, Cpost, ba, cur, s->w, s->to_new, L);
        }
        if (rigid) {
            if (tape) tape->push(TS_SHAPE, cur);
            launch_shape_matching(st, Cpost, s->rigid, cur, s->to_new, L);
            if (tape) tape->recs.back().aux = tape->snap4(s->rigid.rot, (size_t)s->rigid.num_bodies);
        }
        if (immov) {
            if (tape) tape->push(TS_IMMOVABLE, cur);
            launch_immovable(st, Cpost, s->nimm, s->imm, s->to_new, s->Xs, cur, L);
        }
    }
    if (!committed) {
        if (tape) tape->push(TS_COMMIT, cur);
        launch_commit(st, Cpost, cur, s->Xs, s->Vs, s->orig_s, s->Xc, s->Vc, s->orig_c, L);
    }
    s->Pcur = cur;

    const bool post_ab = C.use_vort || C.use_akinci;
    if (tape && post_ab) tape->push(TS_POST_AB, s->Vc);
    if (tape && !post_ab && C.use_xsph) {
        tape->push(TS_XSPH, s->Vc);
        tape->recs.back().aux1 = tape->snap1(s->rho);  // the density textbook XSPH weighs with
    }
    // The post passes keep class positions in their lists where lambda left
    // its densities in class order (SimConsts::cls_post); the velocities are
    // gathered into class order with the positions.
    const bool post_slots = classes && lists && post_ab && fluid && iterations > 0 && !verlet;
    const bool post_planes = walk_planes && post_ab;
    if ((post_ab || C.use_xsph) && classes)  // the post passes read the same positions
        launch_class_refresh(st, s->n, cur, ca, L, post_slots ? s->Vc : nullptr, post_planes ? s->walk_xyz : nullptr,
                             s->walk_stride);
    else if (post_planes)
        launch_walk_planes(st, s->n, cur, s->walk_xyz, s->walk_stride, L);
    if (post_ab) {
        // pass A records each fluid particle's neighbours for passes B and C
        SimConsts Cl = Cpost;
        if (lists) {
            Cl.nbr = s->nbr;
            Cl.nbr_count = s->nbr_count;
            Cl.nbr_cap = kPostListCap;
        }
        if (post_planes) {
            Cl.walk_xyz = s->walk_xyz;
            Cl.walk_stride = s->walk_stride;
        }
        Cl.cls_post = post_slots ? 1 : 0;
        launch_post_a(st, Cl, cur, s->Vc, s->rho, s->off, s->Om, s->Nm, L);
        launch_post_b(st, Cl, cur, s->Vc, s->Om, s->Nm, s->off, C.use_xsph ? s->Vs : s->Vc, L);
        if (tape) {  // what the passes' adjoint reads: omega, normals, pass B's velocities, density
            TapeRec &r = tape->recs.back();
            r.aux = tape->snap4(s->Om);
            tape->snap4(s->Nm);
            if (C.use_xsph) tape->snap4(s->Vs);
            r.aux1 = tape->snap1(s->rho);
        }
        if (C.use_xsph) launch_post_c(st, Cl, cur, s->Vs, s->off, s->mass, s->rho, s->Vc, L);
    } else if (C.use_xsph) {
        SimConsts Cx = Cpost;  // records its own pairs, then sums over them
        if (lists) {
            Cx.nbr = s->nbr;
            Cx.nbr_count = nullptr;
            Cx.nbr_cap = kPostListCap;
        }
        launch_post_c(st, Cx, cur, s->Vc, s->off, s->mass, s->rho, s->Vs, L);
        cudaMemcpyAsync(s->Vc, s->Vs, (size_t)s->n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
    }
}

static bp_status enqueue_update(bp_solver *s, int nsub, float dt, int iterations, int picked, float3 ppos,
                                float3 pvel, LaunchLog *L, bool walk_stats = false)
{
    const float sdt = dt / (float)nsub;
    SimConsts C = make_consts(s, sdt);
    if (picked >= 0) {  // the picked particle teleports: walk the cells
        C.vl = nullptr;
        C.nl_pos = nullptr;
    }
    if (walk_stats) C.nl_stats = s->nl_stats;
    for (int k = 0; k < nsub; ++k) enqueue_substep(s, C, iterations, picked, ppos, L);
    if (picked >= 0) launch_pick(s->stream, picked, s->to_new, s->Xc, ppos, 0, s->Vc, pvel, L);
    launch_check_finite(s->stream, s->n, s->Xc, s->err, L);
    return BP_OK;
}

extern "C" bp_status bp_solver_update(bp_solver *s, int32_t nsub, float dt, int32_t iterations, int32_t picked,
                                      const float *ppos, const float *pvel)
{
    if (!s) return fail(BP_ERR_INVALID_ARGUMENT, "solver is NULL");
    if (nsub <= 0 || !(dt > 0.f) || iterations < 0)
        return fail(BP_ERR_INVALID_ARGUMENT, "num_substeps > 0, dt > 0 and iterations >= 0 required");
    if (s->n <= 0) return BP_OK;  // particlesolver.cuh:778
    if (picked >= s->n) picked = -1;  // the reference ignores out-of-range picks (:790)
    if (picked >= 0 && !ppos) return fail(BP_ERR_INVALID_ARGUMENT, "picked_position is NULL");
    const float3 pp = ppos ? make_float3(ppos[0], ppos[1], ppos[2]) : make_float3(0.f, 0.f, 0.f);
    const float3 pv = pvel ? make_float3(pvel[0], pvel[1], pvel[2]) : make_float3(0.f, 0.f, 0.f);
    if (s->tape) {
        const bp_status st = tape_record_update(s, nsub, dt, iterations, picked, pp, pv);
        if (st != BP_OK) return st;
    }
    LaunchLog L;
    L.stream = s->stream;
    if (picked >= 0) {
        enqueue_update(s, nsub, dt, iterations, picked, pp, pv, &L);
        BP_CUDA(cudaGetLastError());
        s->last_launches = L.count;
        return BP_OK;
    }
    const bool hit = s->exec && s->g_sub == nsub && s->g_iter == iterations && s->g_dt == dt &&
                     s->g_params_version == s->params_version;
    if (!hit) {
        if (s->exec) {
            cudaGraphExecDestroy(s->exec);
            s->exec = nullptr;
        }
        cudaGraph_t g = nullptr;
        BP_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_update(s, nsub, dt, iterations, -1, pp, pv, &L);
        cudaError_t e = cudaStreamEndCapture(s->stream, &g);
        if (e != cudaSuccess) return fail(BP_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&s->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(BP_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        s->g_sub = nsub;
        s->g_iter = iterations;
        s->g_dt = dt;
        s->g_params_version = s->params_version;
        s->graph_launches = L.count;
    }
    BP_CUDA(cudaGraphLaunch(s->exec, s->stream));
    s->last_launches = s->graph_launches;
    return BP_OK;
}

extern "C" bp_status bp_solver_profile(bp_solver *s, int32_t nsub, float dt, int32_t iterations,
                                       int32_t capacity, bp_stage_time *out, int32_t *count)
{
    if (!s || !count || capacity < 0 || (capacity > 0 && !out)) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (s->tape) return fail(BP_ERR_INVALID_ARGUMENT, "not available while a tape records");
    if (nsub <= 0 || !(dt > 0.f) || iterations < 0) return fail(BP_ERR_INVALID_ARGUMENT, "bad step arguments");
    *count = 0;
    if (s->n <= 0) return BP_OK;
    const int maxev = 4096;
    std::vector<cudaEvent_t> ev(maxev + 1);
    std::vector<const char *> names(maxev);
    for (auto &e : ev) BP_CUDA(cudaEventCreate(&e));
    LaunchLog L;
    L.stream = s->stream;
    L.events = ev.data() + 1;
    L.names = names.data();
    L.max_events = maxev;
    BP_CUDA(cudaEventRecord(ev[0], s->stream));
    enqueue_update(s, nsub, dt, iterations, -1, make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f), &L);
    BP_CUDA(cudaStreamSynchronize(s->stream));
    std::vector<bp_stage_time> agg;
    for (int k = 0; k < L.num_events; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
        bool found = false;
        for (auto &a : agg)
            if (!strcmp(a.name, names[k])) {
                a.total_ms += ms;
                a.launches += 1;
                found = true;
            }
        if (!found) {
            bp_stage_time t;
            memset(&t, 0, sizeof(t));
            strncpy(t.name, names[k], sizeof(t.name) - 1);
            t.total_ms = ms;
            t.launches = 1;
            agg.push_back(t);
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    const int m = (int)agg.size() < capacity ? (int)agg.size() : capacity;
    for (int k = 0; k < m; ++k) out[k] = agg[k];
    *count = (int)agg.size();
    s->last_launches = L.count;
    return BP_OK;
}

extern "C" bp_status bp_solver_walk_stats(bp_solver *s, int32_t nsub, float dt, int32_t iterations,
                                          uint64_t out_walks[5])
{
    if (!s || !out_walks) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (s->tape) return fail(BP_ERR_INVALID_ARGUMENT, "not available while a tape records");
    if (nsub <= 0 || !(dt > 0.f) || iterations < 0) return fail(BP_ERR_INVALID_ARGUMENT, "bad step arguments");
    for (int k = 0; k < 5; ++k) out_walks[k] = 0;
    if (s->n <= 0) return BP_OK;
    LaunchLog L;
    L.stream = s->stream;
    BP_CUDA(cudaMemsetAsync(s->nl_stats, 0, 5 * sizeof(unsigned), s->stream));
    enqueue_update(s, nsub, dt, iterations, -1, make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f), &L, true);
    unsigned h[5];
    BP_CUDA(cudaMemcpyAsync(h, s->nl_stats, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    BP_CUDA(cudaStreamSynchronize(s->stream));
    for (int k = 0; k < 5; ++k) out_walks[k] = h[k];
    s->last_launches = L.count;
    return BP_OK;
}

extern "C" bp_status bp_solver_step(bp_solver *s, float dt, int32_t nsub, int32_t iterations)
{
    return bp_solver_update(s, nsub, dt, iterations, -1, nullptr, nullptr);
}

extern "C" bp_status bp_solver_query_original_particle_id(bp_solver *s, int32_t sorted_index, int32_t *out)
{
    if (!s || !out) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (sorted_index < 0 || sorted_index >= s->n) return fail(BP_ERR_INVALID_ARGUMENT, "index out of range");
    BP_CUDA(cudaMemcpyAsync(out, s->orig_c + sorted_index, 4, cudaMemcpyDeviceToHost, s->stream));
    BP_CUDA(cudaStreamSynchronize(s->stream));
    return BP_OK;
}

extern "C" bp_status bp_solver_query_new_particle_id(bp_solver *s, int32_t original, int32_t *out)
{
    if (!s || !out) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (original < 0 || original >= s->n) return fail(BP_ERR_INVALID_ARGUMENT, "id out of range");
    BP_CUDA(cudaMemcpyAsync(out, s->to_new + original, 4, cudaMemcpyDeviceToHost, s->stream));
    BP_CUDA(cudaStreamSynchronize(s->stream));
    return BP_OK;
}

extern "C" bp_status bp_solver_get_particle_position(bp_solver *s, int32_t idx, float out[3])
{
    if (!s || !out) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (idx < 0 || idx >= s->n) {  // the reference returns (0,0,0) (particlesolver.cuh:380)
        out[0] = out[1] = out[2] = 0.f;
        return BP_OK;
    }
    float4 v;
    BP_CUDA(cudaMemcpyAsync(&v, s->Xc + idx, sizeof(float4), cudaMemcpyDeviceToHost, s->stream));
    BP_CUDA(cudaStreamSynchronize(s->stream));
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
    return BP_OK;
}

// Host <-> device state copies move 12 bytes per particle and array: the
// (sorted <-> original) permutation and the float4 packing happen on the GPU
// through the solver's staging buffer.
static bp_status copy_xyz(bp_solver *s, const float4 *src, float *dst, int order)
{
    if (!s || !dst) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (order != BP_ORDER_SORTED && order != BP_ORDER_ORIGINAL) return fail(BP_ERR_INVALID_ARGUMENT, "bad order");
    const int n = s->n;
    if (n == 0) return BP_OK;
    launch_gather_xyz(s->stream, n, src, order == BP_ORDER_ORIGINAL ? s->orig_c : nullptr, s->staging);
    BP_CUDA(cudaMemcpyAsync(dst, s->staging, (size_t)n * 12, cudaMemcpyDeviceToHost, s->stream));
    BP_CUDA(cudaStreamSynchronize(s->stream));
    return BP_OK;
}

extern "C" bp_status bp_solver_copy_positions(bp_solver *s, float *host_xyz, int32_t order)
{
    return copy_xyz(s, s ? s->Xc : nullptr, host_xyz, order);
}

extern "C" bp_status bp_solver_copy_velocities(bp_solver *s, float *host_xyz, int32_t order)
{
    return copy_xyz(s, s ? s->Vc : nullptr, host_xyz, order);
}

extern "C" bp_status bp_solver_set_state(bp_solver *s, const float *hx, const float *hv, int32_t order)
{
    if (!s) return fail(BP_ERR_INVALID_ARGUMENT, "solver is NULL");
    if (order != BP_ORDER_SORTED && order != BP_ORDER_ORIGINAL) return fail(BP_ERR_INVALID_ARGUMENT, "bad order");
    if (s->tape && !s->tape_empty()) return fail(BP_ERR_INVALID_ARGUMENT, "the state cannot change while a tape records");
    const int n = s->n;
    if (n == 0) return BP_OK;
    const int *map = order == BP_ORDER_ORIGINAL ? s->to_new : nullptr;
    if (hx) {
        BP_CUDA(cudaMemcpyAsync(s->staging, hx, (size_t)n * 12, cudaMemcpyHostToDevice, s->stream));
        launch_scatter_xyz(s->stream, n, s->staging, map, s->Xc);
    }
    if (hv) {
        BP_CUDA(cudaMemcpyAsync(s->staging + 3 * (size_t)n, hv, (size_t)n * 12, cudaMemcpyHostToDevice, s->stream));
        launch_scatter_xyz(s->stream, n, s->staging + 3 * (size_t)n, map, s->Vc);
    }
    BP_CUDA(cudaStreamSynchronize(s->stream));
    return BP_OK;
}

// Snapshot layout: header, then the state buffers in state_buffers() order.
struct SnapshotHeader {
    char magic[8];        // "BPSNAP1"
    int64_t n, ncells, num_bodies;
    int64_t pcur_is_b;    // which predicted-position buffer the last update ended in
    int64_t payload;      // bytes after the header
};
static const char kSnapMagic[8] = {'B', 'P', 'S', 'N', 'A', 'P', '1', 0};

static size_t snapshot_payload(bp_solver *s)
{
    size_t b = 0;
    for (const auto &kv : state_buffers(s)) b += kv.second;
    return b;
}

extern "C" bp_status bp_solver_snapshot_size(bp_solver *s, size_t *bytes)
{
    if (!s || !bytes) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    *bytes = sizeof(SnapshotHeader) + snapshot_payload(s);
    return BP_OK;
}

extern "C" bp_status bp_solver_snapshot_save(bp_solver *s, void *host, size_t bytes)
{
    if (!s || !host) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (s->tape) return fail(BP_ERR_INVALID_ARGUMENT, "not available while a tape records");
    const size_t payload = snapshot_payload(s);
    if (bytes < sizeof(SnapshotHeader) + payload) return fail(BP_ERR_CAPACITY, "snapshot buffer too small");
    SnapshotHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, kSnapMagic, sizeof(kSnapMagic));
    h.n = s->n;
    h.ncells = (int64_t)s->ncells;
    h.num_bodies = s->rigid.num_bodies;
    h.pcur_is_b = s->Pcur == s->Pb;
    h.payload = (int64_t)payload;
    memcpy(host, &h, sizeof(h));
    char *dst = (char *)host + sizeof(h);
    for (const auto &kv : state_buffers(s)) {
        BP_CUDA(cudaMemcpyAsync(dst, kv.first, kv.second, cudaMemcpyDeviceToHost, s->stream));
        dst += kv.second;
    }
    BP_CUDA(cudaStreamSynchronize(s->stream));
    return BP_OK;
}

extern "C" bp_status bp_solver_snapshot_load(bp_solver *s, const void *host, size_t bytes)
{
    if (!s || !host) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (s->tape) return fail(BP_ERR_INVALID_ARGUMENT, "not available while a tape records");
    SnapshotHeader h;
    if (bytes < sizeof(h)) return fail(BP_ERR_INVALID_ARGUMENT, "not a snapshot (too short)");
    memcpy(&h, host, sizeof(h));
    if (memcmp(h.magic, kSnapMagic, sizeof(kSnapMagic)) != 0) return fail(BP_ERR_INVALID_ARGUMENT, "not a snapshot");
    const size_t payload = snapshot_payload(s);
    if (h.n != s->n || h.ncells != (int64_t)s->ncells || h.num_bodies != s->rigid.num_bodies ||
        h.payload != (int64_t)payload || bytes < sizeof(h) + payload)
        return fail(BP_ERR_INVALID_ARGUMENT, "snapshot of a different scene (particles, grid or rigid bodies differ)");
    const char *src = (const char *)host + sizeof(h);
    for (const auto &kv : state_buffers(s)) {
        BP_CUDA(cudaMemcpyAsync(kv.first, src, kv.second, cudaMemcpyHostToDevice, s->stream));
        src += kv.second;
    }
    BP_CUDA(cudaStreamSynchronize(s->stream));
    s->Pcur = h.pcur_is_b ? s->Pb : s->Pa;
    return BP_OK;
}

extern "C" bp_status bp_solver_field(bp_solver *s, int32_t field, void **ptr, size_t *bytes)
{
    if (!s || !ptr || !bytes) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    const size_t n = (size_t)s->n;
    switch (field) {
    case BP_FIELD_POSITIONS: *ptr = s->Xc; *bytes = n * 16; break;
    case BP_FIELD_NEW_POSITIONS: *ptr = s->Pcur; *bytes = n * 16; break;
    case BP_FIELD_VELOCITIES: *ptr = s->Vc; *bytes = n * 16; break;
    case BP_FIELD_MAP_TO_ORIGINAL: *ptr = s->orig_c; *bytes = n * 4; break;
    case BP_FIELD_MAP_TO_NEW: *ptr = s->to_new; *bytes = n * 4; break;
    case BP_FIELD_LAMBDAS: *ptr = s->lam; *bytes = n * 4; break;
    case BP_FIELD_DENSITIES: *ptr = s->rho; *bytes = n * 4; break;
    case BP_FIELD_SORTED_CELL_IDS: *ptr = s->sorted_keys; *bytes = n * 4; break;
    case BP_FIELD_CELL_OFFSETS: *ptr = s->off; *bytes = (s->ncells + 1) * 4; break;
    case BP_FIELD_RIGID_ROTATIONS: *ptr = s->rigid.rot; *bytes = (size_t)s->rigid.num_bodies * 16; break;
    case BP_FIELD_RIGID_CMS: *ptr = s->rigid.cm; *bytes = (size_t)s->rigid.num_bodies * 16; break;
    case BP_FIELD_INV_SCALED_MASSES: *ptr = s->w; *bytes = n * 4; break;
    default: return fail(BP_ERR_INVALID_ARGUMENT, "unknown field");
    }
    return BP_OK;
}

extern "C" bp_status bp_solver_copy_field(bp_solver *s, int32_t field, void *dst, size_t bytes)
{
    void *p;
    size_t b;
    bp_status st = bp_solver_field(s, field, &p, &b);
    if (st != BP_OK) return st;
    if (!dst || bytes < b) return fail(BP_ERR_INVALID_ARGUMENT, "destination too small");
    if (b == 0) return BP_OK;
    BP_CUDA(cudaMemcpyAsync(dst, p, b, cudaMemcpyDeviceToHost, s->stream));
    BP_CUDA(cudaStreamSynchronize(s->stream));
    return BP_OK;
}

extern "C" bp_status bp_solver_pack_particle_infos(bp_solver *s, void *device_out)
{
    if (!s || (!device_out && s->n > 0)) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    launch_pack_infos(s->stream, s->n, s->Xc, s->Vc, device_out);
    BP_CUDA(cudaGetLastError());
    return BP_OK;
}

extern "C" bp_status bp_solver_device_errors(bp_solver *s, uint32_t *out)
{
    if (!s || !out) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    unsigned v = 0;
    BP_CUDA(cudaMemcpyAsync(&v, s->err, 4, cudaMemcpyDeviceToHost, s->stream));
    BP_CUDA(cudaMemsetAsync(s->err, 0, 4, s->stream));
    BP_CUDA(cudaStreamSynchronize(s->stream));
    *out = v;
    return BP_OK;
}

extern "C" bp_status bp_solver_last_launch_count(bp_solver *s, int64_t *out)
{
    if (!s || !out) return fail(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = s->last_launches;
    return BP_OK;
}

// ---- stand-alone grid -------------------------------------------------------

extern "C" bp_status bp_grid_workspace_size(int32_t n, int32_t D, size_t *bytes)
{
    if (!bytes || n < 0 || !is_pow2(D) || D < 4 || D > 1024) return fail(BP_ERR_INVALID_ARGUMENT, "bad argument");
    *bytes = sort_scratch_bytes(n > 0 ? n : 1, D);
    return BP_OK;
}

extern "C" bp_status bp_grid_build(void *stream, int32_t n, const float *pos, float cell, int32_t D, int32_t *cell_ids,
                                   int32_t *sorted_cell_ids, int32_t *sorted_ids, int32_t *start, int32_t *end,
                                   void *ws, size_t ws_bytes)
{
    if (n < 0 || !is_pow2(D) || D < 4 || D > 1024 || !(cell > 0.f))
        return fail(BP_ERR_INVALID_ARGUMENT, "bad argument");
    if (n == 0) return BP_OK;
    if (!pos || !cell_ids || !sorted_cell_ids || !sorted_ids || !start || !end || !ws)
        return fail(BP_ERR_INVALID_ARGUMENT, "NULL buffer");
    if (ws_bytes < sort_scratch_bytes(n, D)) return fail(BP_ERR_INVALID_ARGUMENT, "workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    SortScratch sc;
    sort_scratch_carve(ws, n, D, &sc);
    LaunchLog L;
    L.stream = st;
    launch_hash_f3(st, n, pos, cell, D, cell_ids, sc.hist, &L);
    radix_sort_pairs(st, n, D, cell_ids, nullptr, sorted_cell_ids, sorted_ids, sc, true, &L);
    launch_find_start_end(st, n, sorted_cell_ids, start, end, &L);
    BP_CUDA(cudaGetLastError());
    return BP_OK;
}

extern "C" bp_status bp_grid_reset(void *stream, int32_t n, const int32_t *sorted, int32_t *start, int32_t *end)
{
    if (n < 0) return fail(BP_ERR_INVALID_ARGUMENT, "n < 0");
    if (n == 0) return BP_OK;
    if (!sorted || !start || !end) return fail(BP_ERR_INVALID_ARGUMENT, "NULL buffer");
    LaunchLog L;
    L.stream = (cudaStream_t)stream;
    launch_reset_start_end((cudaStream_t)stream, n, sorted, start, end, &L);
    BP_CUDA(cudaGetLastError());
    return BP_OK;
}

extern "C" bp_status bp_grid_neighbor_counts(void *stream, int32_t n, const float *sorted_pos, float cell, int32_t D,
                                             float h, const int32_t *start, const int32_t *end, int32_t *counts)
{
    if (n < 0 || !is_pow2(D) || D < 4 || D > 1024 || !(cell > 0.f) || !(h > 0.f))
        return fail(BP_ERR_INVALID_ARGUMENT, "bad argument");
    if (n == 0) return BP_OK;
    if (!sorted_pos || !start || !end || !counts) return fail(BP_ERR_INVALID_ARGUMENT, "NULL buffer");
    launch_neighbor_counts_f3((cudaStream_t)stream, n, sorted_pos, cell, D, h, start, end, counts);
    BP_CUDA(cudaGetLastError());
    return BP_OK;
}

extern "C" const char *bp_last_error_string(void) { return g_err.c_str(); }

extern "C" int32_t bp_abi_version(void) { return BP_ABI_VERSION; }
