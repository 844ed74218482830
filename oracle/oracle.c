/*
 * oracle.c -- CPU restatement of brass-pan's unified particle solver step.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Each function restates one
 * reference kernel or host step and cites it; paths are inside the brass-pan
 * project, `PS` = brasstower/particlesolver.cuh, `K/` = brasstower/kernel/.
 * The arithmetic keeps the reference's fp32 expression order (compile with
 * -ffp-contract=off) so that, single-threaded, it agrees with the reference's
 * own kernels run on the host (oracle/_ref) to the last bit wherever the
 * reference itself is deterministic.
 *
 * BP_MODE_TEXTBOOK switches the documented reference quirks off (density over
 * all neighbours, exact lambda denominator, s_corr active, no per-pair clamp,
 * gather-only position correction, wind relative to a wind vector).
 */
#include "oracle.h"

#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* One source, two precisions: `real` is float (the restatement, bit-exact to
 * the reference) or, built with ORACLE_REAL_DOUBLE, double (the FP64 host
 * oracle: every state array, parameter copy and operation in double; the
 * reference's float literals keep their float values).  <tgmath.h> makes
 * sqrt, pow, sin, cos, acos and fabs follow the argument type, so the float
 * build calls sqrtf & co. exactly as before. */
typedef or_real real;
#include <tgmath.h>

static int g_threads = 1;
void or_set_threads(int t) { g_threads = t > 0 ? t : 1; }
int or_get_threads(void) { return g_threads; }

/* ---- vector helpers (same operation order as the reference's float3
 * operators: component-wise, dot = x*x' + y*y' + z*z' left to right) ---- */

typedef struct { real x, y, z; } f3;
typedef struct { real x, y, z, w; } f4;

static inline f3 v3(real x, real y, real z) { f3 r = {x, y, z}; return r; }
static inline f3 vadd(f3 a, f3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 vsub(f3 a, f3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 vmul(f3 a, real s) { return v3(a.x * s, a.y * s, a.z * s); }   /* float3 * scalar */
static inline f3 smul(real s, f3 a) { return v3(s * a.x, s * a.y, s * a.z); }   /* scalar * float3 */
static inline f3 vdiv(f3 a, real s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline f3 vneg(f3 a) { return v3(-a.x, -a.y, -a.z); }
static inline real vdot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f3 vcross(f3 a, f3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline real vlen2(f3 a) { return vdot(a, a); }
static inline real vlen(f3 a) { return sqrt(vdot(a, a)); }
/* normalize with rsqrt = 1/sqrt, the host form of the reference's helper */
static inline f3 vnormalize(f3 a) { real inv = 1.0f / sqrt(vdot(a, a)); return vmul(a, inv); }
static inline real fminf_(real a, real b) { return a < b ? a : b; }
static inline real fmaxf_(real a, real b) { return a > b ? a : b; }

static inline void atomic_add3(f3 *arr, int i, f3 d)
{
#pragma omp atomic
    arr[i].x += d.x;
#pragma omp atomic
    arr[i].y += d.y;
#pragma omp atomic
    arr[i].z += d.z;
}

/* ---- SPH kernels (K/fluid.cuh:11-74) --------------------------------------- */

typedef struct {
    real c1, c2, c3, c4, h, h2, half_h;
} sph_consts;

/* SetKernelRadius (K/fluid.cuh:11-27): pi is the literal 3.141592.  Textbook
 * mode scales the Akinci spline's inner offset h^6/64 by the spline constant
 * as in Akinci et al. 2013 (the reference leaves it unscaled, quirk Q7). */
static sph_consts make_sph(real h, int textbook)
{
    sph_consts k;
    k.c1 = 315.f / 64.f / 3.141592f / pow(h, 9.0f);
    k.c2 = -45.f / 3.141592f / pow(h, 6.f);
    k.c3 = 32.0f / 3.141592f / pow(h, 9.f);
    k.c4 = pow(h, 6.0f) / 64.0f;
    if (textbook) k.c4 = k.c3 * k.c4;
    k.h2 = h * h;
    k.half_h = h * 0.5f;
    k.h = h;
    return k;
}

static inline real poly6(const sph_consts *k, real r2) /* K/fluid.cuh:31-43 */
{
    const real t = k->h2 - r2;
    return k->c1 * t * t * t;
}

static inline f3 spiky_grad(const sph_consts *k, f3 v, real r2) /* K/fluid.cuh:45-57 */
{
    const real r = sqrt(r2);
    const real t = k->h - r;
    return vdiv(smul(k->c2 * t * t, v), r);
}

static inline real akinci_spline(const sph_consts *k, real r) /* K/fluid.cuh:59-74 (quirk Q7 kept) */
{
    const real t = (k->h - r) * r;
    const real t3 = t * t * t;
    if (r >= k->half_h) return k->c3 * t3;
    return 2.0f * k->c3 * t3 - k->c4;
}

/* ---- hash grid (K/grid.cuh) -------------------------------------------------- */

typedef struct { int x, y, z; } i3;

/* calcGridPos, K/grid.cuh:9-13.  The cell of a position is integer work that
 * the reference defines in float arithmetic (p + 50000 keeps about 0.004 m of
 * resolution), so both precisions compute it in float from the position
 * rounded to float: the FP64 oracle then builds the grid the fp32 step builds
 * and differs from it only in the floating-point sums. */
static inline i3 grid_pos(f3 p, real cell)
{
    const float cf = (float)cell;
    i3 c;
    c.x = (int)(((float)p.x + 50000.0f) / cf);
    c.y = (int)(((float)p.y + 50000.0f) / cf);
    c.z = (int)(((float)p.z + 50000.0f) / cf);
    return c;
}

static inline int grid_addr(int x, int y, int z, int D) /* calcGridAddress, K/grid.cuh:15-22 */
{
    const unsigned m = (unsigned)D - 1u;
    const unsigned cx = (unsigned)x & m, cy = (unsigned)y & m, cz = (unsigned)z & m;
    return (int)(cx * ((unsigned)D * (unsigned)D) + cy * (unsigned)D + cz);
}

/* Stable sort of [0,n) by key: LSD radix sort, 3 passes of 11 bits (keys are
 * non-negative and below 2^31).  Replaces cub::DeviceRadixSort::SortPairs
 * (PS:721-738), which is also a stable LSD radix sort. */
static void stable_sort_by_key(int n, const int *keys, int *order)
{
    int *tmp = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int *cnt = (int *)malloc(sizeof(int) * 2049);
    for (int i = 0; i < n; ++i) order[i] = i;
    for (int pass = 0; pass < 3; ++pass) {
        const int shift = 11 * pass;
        memset(cnt, 0, sizeof(int) * 2049);
        for (int i = 0; i < n; ++i) cnt[(((unsigned)keys[order[i]]) >> shift & 2047u) + 1]++;
        for (int d = 0; d < 2048; ++d) cnt[d + 1] += cnt[d];
        for (int i = 0; i < n; ++i) tmp[cnt[((unsigned)keys[order[i]]) >> shift & 2047u]++] = order[i];
        memcpy(order, tmp, sizeof(int) * (size_t)n);
    }
    free(tmp);
    free(cnt);
}

/* findStartEndId (K/grid.cuh:70-99) */
static void find_start_end(int n, const int *sorted, int *start, int *end)
{
    for (int i = 0; i < n; ++i) {
        const int u = sorted[i];
        if (i > 0) {
            const int v = sorted[i - 1];
            if (u != v) { start[u] = i; end[v] = i; }
        } else {
            start[u] = i;
        }
        if (i == n - 1) end[u] = n;
    }
}

/* resetStartEndId (K/grid.cuh:101-132) */
static void reset_start_end(int n, const int *sorted, int *start, int *end)
{
    for (int i = 0; i < n; ++i) {
        start[sorted[i]] = -1;
        end[sorted[i]] = -1;
    }
}

int or_grid_build(int n, const float *pos, float cell, int D, int *cell_ids, int *sorted_cell_ids,
                  int *sorted_particle_ids, int *cell_start, int *cell_end)
{
    for (int i = 0; i < n; ++i) { /* updateGridId, K/grid.cuh:30-47 */
        const i3 c = grid_pos(v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), cell);
        cell_ids[i] = grid_addr(c.x, c.y, c.z, D);
    }
    stable_sort_by_key(n, cell_ids, sorted_particle_ids);
    for (int i = 0; i < n; ++i) sorted_cell_ids[i] = cell_ids[sorted_particle_ids[i]];
    find_start_end(n, sorted_cell_ids, cell_start, cell_end);
    return 0;
}

int or_neighbor_counts(int n, const float *sp, float cell, int D, float h, const int *cs,
                       const int *ce, int *counts)
{
    const real h2 = h * h;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < n; ++i) {
        const f3 pi = v3(sp[3 * i], sp[3 * i + 1], sp[3 * i + 2]);
        const i3 c = grid_pos(pi, cell);
        int cnt = 0;
        for (int z = c.z - 1; z <= c.z + 1; z++)
            for (int y = c.y - 1; y <= c.y + 1; y++)
                for (int x = c.x - 1; x <= c.x + 1; x++) {
                    const int a = grid_addr(x, y, z, D);
                    for (int j = cs[a]; j < ce[a]; j++) {
                        const f3 pj = v3(sp[3 * j], sp[3 * j + 1], sp[3 * j + 2]);
                        if (vlen2(vsub(pi, pj)) <= h2) cnt++;
                    }
                }
        counts[i] = cnt;
    }
    return 0;
}

/* ---- solver state ------------------------------------------------------------ */

struct or_solver {
    int n, D, nb, npairs, nfaces, nimm, nplanes, nbend;
    bp_params prm;
    real wind[3]; /* prm.wind_velocity, or an override in this precision (or_set_wind) */
    f3 *x, *p, *v, *sx, *sp, *sv, *dX, *tmp, *omega, *normal;
    real *m, *sm, *w, *lambda, *rho;
    int *phase, *sphase, *group, *sgroup, *to_orig, *sto_orig, *to_new;
    int *cell_id, *sorted_cell, *sorted_pid, *cell_start, *cell_end;
    int *ranges, *pairs, *faces, *imm, *bends;
    real *dparams, *planes;
    f3 *rest, *cms;
    f4 *rot;
};

#define ALLOC(ptr, count) ((ptr) = calloc((size_t)((count) > 0 ? (count) : 1), sizeof(*(ptr))))

or_solver *or_create(const bp_scene_desc *sc, const bp_params *prm)
{
    or_solver *s = (or_solver *)calloc(1, sizeof(or_solver));
    const int n = sc->num_particles;
    s->n = n;
    s->prm = *prm;
    for (int q = 0; q < 3; ++q) s->wind[q] = prm->wind_velocity[q];
    s->D = prm->grid_dim;
    ALLOC(s->x, n); ALLOC(s->p, n); ALLOC(s->v, n); ALLOC(s->sx, n); ALLOC(s->sp, n); ALLOC(s->sv, n);
    ALLOC(s->dX, n); ALLOC(s->tmp, n); ALLOC(s->omega, n); ALLOC(s->normal, n);
    ALLOC(s->m, n); ALLOC(s->sm, n); ALLOC(s->w, n); ALLOC(s->lambda, n); ALLOC(s->rho, n);
    ALLOC(s->phase, n); ALLOC(s->sphase, n); ALLOC(s->group, n); ALLOC(s->sgroup, n);
    ALLOC(s->to_orig, n); ALLOC(s->sto_orig, n); ALLOC(s->to_new, n);
    ALLOC(s->cell_id, n); ALLOC(s->sorted_cell, n); ALLOC(s->sorted_pid, n);
    const size_t cells = (size_t)s->D * s->D * s->D;
    s->cell_start = (int *)malloc(cells * sizeof(int));
    s->cell_end = (int *)malloc(cells * sizeof(int));
    for (size_t c = 0; c < cells; ++c) { s->cell_start[c] = -1; s->cell_end[c] = -1; }
    for (int i = 0; i < n; ++i) {
        s->x[i] = v3(sc->positions[3 * i], sc->positions[3 * i + 1], sc->positions[3 * i + 2]);
        s->p[i] = s->x[i];
        s->v[i] = sc->velocities ? v3(sc->velocities[3 * i], sc->velocities[3 * i + 1], sc->velocities[3 * i + 2])
                                 : v3(0, 0, 0);
        s->m[i] = sc->masses[i];
        s->phase[i] = sc->phases[i];
        s->group[i] = sc->group_ids ? sc->group_ids[i] : 0;
        s->to_orig[i] = i;
        s->to_new[i] = i;
    }
    s->nplanes = sc->num_planes;
    ALLOC(s->planes, 6 * s->nplanes);
    for (int q = 0; q < 6 * s->nplanes; ++q) s->planes[q] = sc->planes[q];
    s->npairs = sc->num_distance_constraints;
    ALLOC(s->pairs, 2 * s->npairs);
    ALLOC(s->dparams, 2 * s->npairs);
    if (s->npairs > 0) {
        memcpy(s->pairs, sc->distance_pairs, sizeof(int) * 2 * (size_t)s->npairs);
        for (int q = 0; q < 2 * s->npairs; ++q) s->dparams[q] = sc->distance_params[q];
    }
    s->nfaces = sc->num_wind_faces;
    ALLOC(s->faces, 3 * s->nfaces);
    if (s->nfaces) memcpy(s->faces, sc->wind_faces, sizeof(int) * 3 * (size_t)s->nfaces);
    s->nb = sc->num_rigid_bodies;
    ALLOC(s->ranges, 2 * s->nb);
    if (s->nb) memcpy(s->ranges, sc->rigid_ranges, sizeof(int) * 2 * (size_t)s->nb);
    ALLOC(s->rest, n);
    if (sc->rigid_rest_positions)
        for (int i = 0; i < n; ++i)
            s->rest[i] = v3(sc->rigid_rest_positions[3 * i], sc->rigid_rest_positions[3 * i + 1],
                            sc->rigid_rest_positions[3 * i + 2]);
    ALLOC(s->rot, s->nb);
    ALLOC(s->cms, s->nb);
    for (int b = 0; b < s->nb; ++b) { s->rot[b].x = s->rot[b].y = s->rot[b].z = 0.f; s->rot[b].w = 1.f; }
    s->nimm = sc->num_immovables;
    ALLOC(s->imm, s->nimm);
    if (s->nimm) memcpy(s->imm, sc->immovables, sizeof(int) * (size_t)s->nimm);
    s->nbend = sc->num_bendings;
    ALLOC(s->bends, 4 * s->nbend);
    if (s->nbend) memcpy(s->bends, sc->bendings, sizeof(int) * 4 * (size_t)s->nbend);
    return s;
}

void or_destroy(or_solver *s)
{
    if (!s) return;
    void *ptrs[] = {s->x, s->p, s->v, s->sx, s->sp, s->sv, s->dX, s->tmp, s->omega, s->normal, s->m, s->sm,
                    s->w, s->lambda, s->rho, s->phase, s->sphase, s->group, s->sgroup, s->to_orig,
                    s->sto_orig, s->to_new, s->cell_id, s->sorted_cell, s->sorted_pid, s->cell_start,
                    s->cell_end, s->ranges, s->pairs, s->faces, s->imm, s->dparams, s->planes, s->rest,
                    s->cms, s->rot, s->bends};
    for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); ++k) free(ptrs[k]);
    free(s);
}

int or_set_params(or_solver *s, const bp_params *prm)
{
    if (prm->grid_dim != s->D) return 1;
    s->prm = *prm;
    for (int q = 0; q < 3; ++q) s->wind[q] = prm->wind_velocity[q];
    return 0;
}

int or_real_size(void) { return (int)sizeof(real); }

int or_set_wind(or_solver *s, const real *wind)
{
    for (int q = 0; q < 3; ++q) s->wind[q] = wind[q];
    return 0;
}

int or_set_distance_params(or_solver *s, const real *params)
{
    for (int q = 0; q < 2 * s->npairs; ++q) s->dparams[q] = params[q];
    return 0;
}

int or_set_state(or_solver *s, const real *x, const real *v)
{
    for (int i = 0; i < s->n; ++i) {
        if (x) s->x[i] = v3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
        if (v) s->v[i] = v3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    }
    return 0;
}

/* Adopts a complete state in another solver's sorted arrangement: positions
 * and velocities [N][3] in that order, its sorted->original map, and
 * optionally the rigid-body quaternions [B][4]; per-particle constants follow
 * the new arrangement.  Used to restart both solvers from identical inputs. */
int or_set_full_state(or_solver *s, const real *x, const real *v, const int *to_orig, const real *rot)
{
    const int n = s->n;
    real *m0 = (real *)malloc(sizeof(real) * (size_t)(n > 0 ? n : 1));
    int *ph0 = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int *g0 = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) {
        m0[s->to_orig[i]] = s->m[i];
        ph0[s->to_orig[i]] = s->phase[i];
        g0[s->to_orig[i]] = s->group[i];
    }
    for (int i = 0; i < n; ++i) {
        const int o = to_orig[i];
        s->to_orig[i] = o;
        s->to_new[o] = i;
        s->m[i] = m0[o];
        s->phase[i] = ph0[o];
        s->group[i] = g0[o];
        s->x[i] = v3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
        s->v[i] = v3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    }
    if (rot)
        for (int b = 0; b < s->nb; ++b) {
            s->rot[b].x = rot[4 * b];
            s->rot[b].y = rot[4 * b + 1];
            s->rot[b].z = rot[4 * b + 2];
            s->rot[b].w = rot[4 * b + 3];
        }
    free(m0);
    free(ph0);
    free(g0);
    return 0;
}

#define SWAP(a, b) do { void *t_ = (void *)(a); (a) = (b); (b) = t_; } while (0)

/* updateGrid (PS:712-765): hash, stable sort, start/end, 7-array reorder */
static void update_grid(or_solver *s)
{
    const int n = s->n, D = s->D;
    const real cell = s->prm.cell_size;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < n; ++i) {
        const i3 c = grid_pos(s->p[i], cell);
        s->cell_id[i] = grid_addr(c.x, c.y, c.z, D);
    }
    stable_sort_by_key(n, s->cell_id, s->sorted_pid);
    for (int i = 0; i < n; ++i) s->sorted_cell[i] = s->cell_id[s->sorted_pid[i]];
    find_start_end(n, s->sorted_cell, s->cell_start, s->cell_end);
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < n; ++i) { /* reorderParticlesData, K/grid.cuh:134-163 */
        const int o = s->sorted_pid[i];
        s->sp[i] = s->p[o];
        s->sx[i] = s->x[o];
        s->sv[i] = s->v[o];
        s->sm[i] = s->m[o];
        s->sphase[i] = s->phase[o];
        s->sto_orig[i] = s->to_orig[o];
        s->sgroup[i] = s->group[o];
    }
    SWAP(s->sp, s->p); SWAP(s->sx, s->x); SWAP(s->sv, s->v); SWAP(s->sm, s->m);
    SWAP(s->sphase, s->phase); SWAP(s->sto_orig, s->to_orig); SWAP(s->sgroup, s->group);
}

/* The 27-cell neighbourhood walk of every scan kernel (e.g. K/fluid.cuh:104-141):
 * cells around the CURRENT position's cell, z outer, x inner, j ascending. */
#define FOR_EACH_CANDIDATE(S, PI, J)                                                     \
    for (int dz_ = -1; dz_ <= 1; ++dz_)                                                  \
        for (int dy_ = -1; dy_ <= 1; ++dy_)                                              \
            for (int dx_ = -1; dx_ <= 1; ++dx_)                                          \
                for (int a_ = grid_addr(c_.x + dx_, c_.y + dy_, c_.z + dz_, (S)->D),     \
                         J = (S)->cell_start[a_], e_ = (S)->cell_end[a_];                \
                     J < e_; ++J)

static inline f3 plane_o(const or_solver *s, int k) { return v3(s->planes[6 * k], s->planes[6 * k + 1], s->planes[6 * k + 2]); }
static inline f3 plane_n(const or_solver *s, int k) { return v3(s->planes[6 * k + 3], s->planes[6 * k + 4], s->planes[6 * k + 5]); }

/* planeStabilize (K/particleplane.cuh:3-19), both x and p move */
static void plane_stabilize(or_solver *s, f3 o, f3 nrm, real r)
{
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < s->n; ++i) {
        const real d = vdot(vsub(o, s->x[i]), nrm) + r;
        if (d <= 0) continue;
        s->x[i] = vadd(s->x[i], smul(d, nrm));
        s->p[i] = vadd(s->p[i], smul(d, nrm));
    }
}

/* particlePlaneCollisionConstraint (K/particleplane.cuh:21-58), friction per
 * Macklin et al. 2014 eq. 24 with the reference's static/dynamic constants */
static void plane_collision(or_solver *s, f3 o, f3 nrm, real r)
{
    const real fs = s->prm.friction_static, fd = s->prm.friction_dynamic;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < s->n; ++i) {
        const real d = vdot(vsub(o, s->p[i]), nrm) + r;
        if (d <= 0) continue;
        const f3 x = s->x[i];
        const f3 diff = vsub(s->p[i], x);
        const real dn = vdot(diff, nrm);
        const f3 dt = vsub(diff, smul(dn, nrm));
        const real dtl = vlen(dt);
        const f3 resolved = vadd(smul(d, nrm), s->p[i]);
        const f3 dx = vsub(resolved, x);
        const f3 tdx = vsub(dx, smul(vdot(dx, nrm), nrm));
        if (dtl < fs * dn)
            s->p[i] = vsub(resolved, tdx);
        else
            s->p[i] = vsub(resolved, vmul(tdx, fminf_(fd * -dn / dtl, 1.0f)));
    }
}

/* particleParticleCollisionConstraint (K/particleparticle.cuh:5-101) -> dX */
static void particle_collision(or_solver *s, real radius)
{
    const int n = s->n;
    const real fs = s->prm.friction_static, fd = s->prm.friction_dynamic;
    const real cell = s->prm.cell_size;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < n; ++i) {
        const f3 xi = s->x[i];
        const f3 xip = s->p[i];
        f3 sum_d = v3(0, 0, 0), sum_f = v3(0, 0, 0);
        const real wi = s->w[i];
        const i3 c_ = grid_pos(xip, cell);
        const int phi = s->phase[i];
        int count = 0;
        FOR_EACH_CANDIDATE(s, xip, j) {
            const int phj = s->phase[j];
            if (!(i != j && phi != phj && (phi > 0 || phj > 0))) continue;
            const f3 xjp = s->p[j];
            const f3 diff = vsub(xip, xjp);
            const real d2 = vlen2(diff);
            if (!(d2 < radius * radius * 4.0f && d2 > 1e-5f)) continue;
            const real dist = sqrt(d2);
            const real wj = s->w[j];
            const real w1 = wi / (wi + wj);
            const real w2 = wj / (wi + wj);
            const f3 proj = vmul(diff, 2.0f * radius / dist - 1.0f);
            const f3 dxi = smul(w1, proj);
            const f3 xistar = vadd(dxi, xip);
            sum_d = vadd(sum_d, dxi);
            const f3 dxj = smul(-w2, proj);
            const real dxi2 = vlen2(dxi);
            if (dxi2 > radius * radius * 0.001f * 0.001f) {
                count += 1;
                const f3 xj = s->x[j];
                const f3 xjstar = vadd(dxj, xjp);
                const f3 t1 = vsub(vsub(xistar, xi), vsub(xjstar, xj));
                const f3 nn = vdiv(diff, dist);
                const f3 tdx = vsub(t1, smul(vdot(t1, nn), nn));
                const real tl2 = vlen2(tdx);
                if (tl2 <= (fs * fs) * dxi2)
                    sum_f = vsub(sum_f, smul(w1, tdx));
                else
                    sum_f = vsub(sum_f, vmul(smul(w1, tdx), fminf_(fd * sqrt(dxi2 / tl2), 1.0f)));
            }
        }
        if (count == 0)
            atomic_add3(s->dX, i, sum_d);
        else
            atomic_add3(s->dX, i, vadd(sum_d, vdiv(sum_f, (real)count)));
    }
}

/* fluidLambda (K/fluid.cuh:78-159).  Reference mode: density over j >= i
 * (sorted index, Q1), solid neighbours scaled, lambda = -C/denominator (Q2).
 * Textbook mode: all neighbours, lambda = -C/(sum|grad C|^2 + eps). */
static void fluid_lambda(or_solver *s, const sph_consts *k)
{
    const int n = s->n;
    const real rho0 = s->prm.rest_density, solid = s->prm.solid_density_scale;
    const int textbook = s->prm.mode == BP_MODE_TEXTBOOK;
    const int clampC = (s->prm.stage_mask & BP_STAGE_AKINCI) != 0;
    const real cell = s->prm.cell_size;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < n; ++i) {
        if (s->phase[i] > 0) continue;
        const f3 pi = s->p[i];
        real density = 0.f, sum_g2 = 0.f;
        f3 grad_i = v3(0, 0, 0);
        const i3 c_ = grid_pos(pi, cell);
        FOR_EACH_CANDIDATE(s, pi, j) {
            if (!textbook && !(i <= j)) continue;
            const f3 pj = s->p[j];
            const f3 diff = vsub(pi, pj);
            const real d2 = vlen2(diff);
            if (d2 <= k->h2) {
                const real mj = s->m[j];
                const real ld = mj * poly6(k, d2);
                density += (s->phase[j] < 0) ? ld : solid * ld;
                if (textbook && d2 > 0) {
                    const f3 g = vdiv(smul(-mj, spiky_grad(k, diff, d2)), rho0);
                    sum_g2 += vdot(g, g);
                    grad_i = vsub(grad_i, g);
                }
            }
        }
        real C = density / rho0 - 1.0f;
        if (clampC) C = fmaxf_(C, 0.0f);
        real lam;
        if (textbook) {
            sum_g2 += vdot(grad_i, grad_i);
            lam = -C / (sum_g2 + s->prm.relaxation);
        } else {
            lam = -C / s->prm.lambda_denominator;
        }
        s->lambda[i] = lam;
        s->rho[i] = density;
    }
}

/* fluidPosition (K/fluid.cuh:161-228) -> dX.  Reference mode: pairs i < j,
 * scatter to both ends with atomics, s_corr only when Akinci is off, per-pair
 * clamp.  Textbook mode: every fluid particle gathers over all neighbours. */
static void fluid_position(or_solver *s, const sph_consts *k)
{
    const int n = s->n;
    const real rho0 = s->prm.rest_density, K = s->prm.scorr_k;
    const int N = s->prm.scorr_n;
    const int textbook = s->prm.mode == BP_MODE_TEXTBOOK;
    const int scorr = textbook || !(s->prm.stage_mask & BP_STAGE_AKINCI);
    const real clampv = textbook ? -1.0f : s->prm.delta_clamp; /* textbook PBF: no per-pair clamp */
    const real wq = poly6(k, pow(s->prm.scorr_dq * k->h, 2.f));
    const real cell = s->prm.cell_size;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < n; ++i) {
        if (s->phase[i] > 0) continue;
        const f3 pi = s->p[i];
        f3 sum = v3(0, 0, 0);
        const i3 c_ = grid_pos(pi, cell);
        const real mi = s->m[i];
        const real li = s->lambda[i];
        const real inv_rho = 1.0f / rho0;
        FOR_EACH_CANDIDATE(s, pi, j) {
            if (textbook ? (i == j) : !(i < j)) continue;
            const f3 pj = s->p[j];
            const f3 diff = vsub(pi, pj);
            const real d2 = vlen2(diff);
            if (d2 <= k->h2 && d2 > 0) {
                const real mj = s->m[j];
                real sl = li + s->lambda[j];
                if (scorr) sl += -K * pow(poly6(k, d2) / wq, (real)N);
                f3 delta = smul(sl, spiky_grad(k, diff, d2));
                if (clampv > 0) {
                    const real len = vlen(delta);
                    delta = (len < clampv) ? delta : vdiv(vmul(delta, fminf_(len, clampv)), len);
                }
                sum = vadd(sum, smul(mj, delta));
                if (!textbook) atomic_add3(s->dX, j, vmul(smul(-mi, delta), inv_rho));
            }
        }
        atomic_add3(s->dX, i, vmul(sum, inv_rho));
    }
}

/* distanceConstraints (K/distance.cuh:3-40) -> dX */
static void distance_constraints(or_solver *s)
{
#pragma omp parallel for num_threads(g_threads)
    for (int c = 0; c < s->npairs; ++c) {
        const int id1 = s->to_new[s->pairs[2 * c]], id2 = s->to_new[s->pairs[2 * c + 1]];
        const real d0 = s->dparams[2 * c], kst = s->dparams[2 * c + 1];
        const f3 x12 = vsub(s->p[id1], s->p[id2]);
        const real d12 = vlen(x12);
        if (d12 <= 1e-5f) continue;
        const f3 nn = vdiv(x12, d12);
        const real w1 = s->w[id1], w2 = s->w[id2];
        const real sw = w1 + w2;
        const f3 kk = vmul(vmul(nn, (d12 - d0) / sw), kst);
        atomic_add3(s->dX, id1, smul(-w1, kk));
        atomic_add3(s->dX, id2, smul(w2, kk));
    }
}

/* bendingConstraints (K/bending.cuh:3-75) -> dX: the dihedral angle of the
 * triangles (1, 2, 3) and (1, 2, 4) over the hinge 1-2 pulled towards pi with
 * the gradients of Mueller et al. 2007 (appendix A), stiffness k (0.8 there). */
static void bending_constraints(or_solver *s, real kb)
{
#pragma omp parallel for num_threads(g_threads)
    for (int c = 0; c < s->nbend; ++c) {
        const int id1 = s->to_new[s->bends[4 * c]], id2 = s->to_new[s->bends[4 * c + 1]];
        const int id3 = s->to_new[s->bends[4 * c + 2]], id4 = s->to_new[s->bends[4 * c + 3]];
        const f3 p1 = s->p[id1];
        const f3 e = vsub(s->p[id2], p1), a = vsub(s->p[id3], p1), b = vsub(s->p[id4], p1);
        const f3 ca = vcross(e, a), cb = vcross(e, b);
        const real la = vlen(ca);
        if (la <= 1e-5f) continue;
        const real lb = vlen(cb);
        if (lb <= 1e-5f) continue;
        const f3 n1 = vmul(ca, 1.0f / la), n2 = vmul(cb, 1.0f / lb);
        real d = vdot(n1, n2);
        d = fminf_(fmaxf_(d, -1.0f), 1.0f);
        const f3 en1 = vcross(e, n1), en2 = vcross(e, n2);
        const f3 an1 = vcross(a, n1), an2 = vcross(a, n2);
        const f3 bn1 = vcross(b, n1), bn2 = vcross(b, n2);
        const f3 q3 = vdiv(vsub(en2, vmul(en1, d)), la);
        const f3 q4 = vdiv(vsub(en1, vmul(en2, d)), lb);
        const f3 q2 = vsub(vdiv(vneg(vsub(an2, vmul(an1, d))), la), vdiv(vsub(bn1, vmul(bn2, d)), lb));
        const f3 q1 = vsub(vsub(vneg(q2), q3), q4);
        const real w1 = s->w[id1], w2 = s->w[id2], w3 = s->w[id3], w4 = s->w[id4];
        const real den = w1 * vlen2(q1) + w2 * vlen2(q2) + w3 * vlen2(q3) + w4 * vlen2(q4);
        const real num = sqrt(1.0f - d * d) * (acos(d) - 3.141592f);
        if (den <= 1e-5f) continue;
        const real sc = num / den;
        atomic_add3(s->dX, id1, vmul(vmul(smul(-w1, q1), sc), kb));
        atomic_add3(s->dX, id2, vmul(vmul(smul(-w2, q2), sc), kb));
        atomic_add3(s->dX, id3, vmul(vmul(smul(-w3, q3), sc), kb));
        atomic_add3(s->dX, id4, vmul(vmul(smul(-w4, q4), sc), kb));
    }
}

/* applyWindForce (K/wind.cuh:3-50) -> dX.  Reference mode uses the face's
 * mean particle velocity (Q5); textbook mode uses it relative to the wind. */
static void wind_force(or_solver *s, real dt)
{
    const int textbook = s->prm.mode == BP_MODE_TEXTBOOK;
    const f3 wind = v3(s->wind[0], s->wind[1], s->wind[2]);
    const real cd = s->prm.wind_drag, cl = s->prm.wind_lift;
#pragma omp parallel for num_threads(g_threads)
    for (int f = 0; f < s->nfaces; ++f) {
        const int id1 = s->to_new[s->faces[3 * f]], id2 = s->to_new[s->faces[3 * f + 1]],
                  id3 = s->to_new[s->faces[3 * f + 2]];
        const f3 p1 = s->p[id1], p2 = s->p[id2], p3 = s->p[id3];
        const f3 a = vsub(p2, p1), b = vsub(p3, p1);
        f3 v = vdiv(vadd(vadd(s->v[id1], s->v[id2]), s->v[id3]), 3.f);
        if (textbook) v = vsub(v, wind);
        const real lv = vlen(v);
        if (lv <= 1e-5f) continue;
        const f3 vh = vdiv(v, lv);
        f3 fnrm = vcross(a, b);
        const real lf = vlen(fnrm);
        if (lf <= 1e-5f) continue;
        fnrm = vdiv(fnrm, lf);
        fnrm = (vdot(fnrm, v) > 0) ? fnrm : vneg(fnrm);
        const real area = 0.5f * lf;
        const f3 drag = smul(cd * (lv * lv) * area * vdot(fnrm, vh), vneg(vh));
        const f3 uh = vcross(vcross(fnrm, vh), vh);
        const f3 lift = smul(cl * (lv * lv) * area * vdot(fnrm, vh), uh);
        const f3 force = vadd(drag, lift);
        const f3 mv = vmul(vmul(force, dt), dt);
        atomic_add3(s->dX, id1, vdiv(mv, s->m[id1]));
        atomic_add3(s->dX, id2, vdiv(mv, s->m[id2]));
        atomic_add3(s->dX, id3, vdiv(mv, s->m[id3]));
    }
}

/* quaternion helpers (brasstower/cuda/cudamatrix.cuh:110-172) */
static inline f4 qmul(f4 a, f4 b)
{
    f4 r;
    r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
    r.y = a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x;
    r.z = a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w;
    r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
    return r;
}
static inline f4 qaxis(f3 d, real angle)
{
    const real sh = sin(angle * 0.5f), ch = cos(angle * 0.5f);
    f4 r = {d.x * sh, d.y * sh, d.z * sh, ch};
    return r;
}
static inline f4 qnormalize(f4 q)
{
    const real inv = 1.0f / sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    f4 r = {q.x * inv, q.y * inv, q.z * inv, q.w * inv};
    return r;
}
typedef struct { f3 c0, c1, c2; } m3;
static inline m3 qmatrix(f4 q)
{
    const real x2 = q.x * q.x, y2 = q.y * q.y, z2 = q.z * q.z;
    m3 m;
    m.c0 = v3(1 - 2 * y2 - 2 * z2, 2 * q.x * q.y + 2 * q.w * q.z, 2 * q.x * q.z - 2 * q.w * q.y);
    m.c1 = v3(2 * q.x * q.y - 2 * q.w * q.z, 1 - 2 * x2 - 2 * z2, 2 * q.y * q.z + 2 * q.w * q.x);
    m.c2 = v3(2 * q.x * q.z + 2 * q.w * q.y, 2 * q.y * q.z - 2 * q.w * q.x, 1 - 2 * x2 - 2 * y2);
    return m;
}
static inline f3 mvmul(m3 m, f3 a)
{
    f3 o = vmul(m.c0, a.x);
    o = vadd(o, vmul(m.c1, a.y));
    o = vadd(o, vmul(m.c2, a.z));
    return o;
}

/* shapeMatchingAlphaOne (K/shapematching.cuh:8-99): unweighted centre of
 * mass, A_pq by columns, warm-started robust rotation extraction (Mueller et
 * al. 2016) with the denominator as written (Q6: 1/|sum| + 1e-9), goal
 * positions written with alpha = 1.  Sums run in particle order (the host
 * build of the reference sums its 64 threads in the same order).  Unlike the
 * reference (at most 64 particles per body) any body size is accepted. */
static void shape_matching(or_solver *s)
{
    const int iters = s->prm.rotation_iterations;
#pragma omp parallel for num_threads(g_threads)
    for (int b = 0; b < s->nb; ++b) {
        const int r0 = s->ranges[2 * b], r1 = s->ranges[2 * b + 1];
        const int np = r1 - r0;
        f3 sum = v3(0, 0, 0);
        for (int t = 0; t < np; ++t) sum = vadd(sum, s->p[s->to_new[r0 + t]]);
        const f3 cm = vdiv(sum, (real)np);
        s->cms[b] = cm;
        f3 a0 = v3(0, 0, 0), a1 = v3(0, 0, 0), a2 = v3(0, 0, 0);
        for (int t = 0; t < np; ++t) {
            const f3 q = s->rest[r0 + t];
            const f3 pc = vsub(s->p[s->to_new[r0 + t]], cm);
            a0 = vadd(a0, vmul(pc, q.x));
            a1 = vadd(a1, vmul(pc, q.y));
            a2 = vadd(a2, vmul(pc, q.z));
        }
        f4 q = s->rot[b];
        for (int it = 0; it < iters; ++it) {
            const m3 R = qmatrix(q);
            const f3 num = vadd(vadd(vcross(R.c0, a0), vcross(R.c1, a1)), vcross(R.c2, a2));
            const real den = 1.0f / fabs(vdot(R.c0, a0) + vdot(R.c1, a1) + vdot(R.c2, a2)) + 1e-9f;
            const f3 om = vmul(num, den);
            const real w2 = vlen2(om);
            if (w2 <= 1e-9f) break;
            const real w = sqrt(w2);
            q = qmul(qaxis(vdiv(om, w), w), q);
            q = qnormalize(q);
        }
        const m3 R = qmatrix(q);
        s->rot[b] = q;
        for (int t = 0; t < np; ++t) s->p[s->to_new[r0 + t]] = vadd(mvmul(R, s->rest[r0 + t]), cm);
    }
}

/* fluidOmega (K/fluid.cuh:231-279) */
static void fluid_omega(or_solver *s, const sph_consts *k)
{
    const real cell = s->prm.cell_size;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < s->n; ++i) {
        const int phi = s->phase[i];
        if (phi >= 0) continue;
        const f3 pi = s->p[i], vi = s->v[i];
        f3 om = v3(0, 0, 0);
        const i3 c_ = grid_pos(pi, cell);
        FOR_EACH_CANDIDATE(s, pi, j) {
            if (!(i != j && phi == s->phase[j])) continue;
            const f3 diff = vsub(pi, s->p[j]);
            const real d2 = vlen2(diff);
            if (d2 <= k->h2 && d2 > 0) om = vadd(om, vcross(vsub(s->v[j], vi), spiky_grad(k, diff, d2)));
        }
        s->omega[i] = om;
    }
}

/* fluidVorticity (K/fluid.cuh:281-336): v updated in place (no mass division, Q9) */
static void fluid_vorticity(or_solver *s, const sph_consts *k, real dt)
{
    const real eps = s->prm.vorticity_eps, cell = s->prm.cell_size;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < s->n; ++i) {
        const int phi = s->phase[i];
        if (phi >= 0) continue;
        const f3 om = s->omega[i], pi = s->p[i];
        f3 eta = v3(0, 0, 0);
        const i3 c_ = grid_pos(pi, cell);
        FOR_EACH_CANDIDATE(s, pi, j) {
            if (!(i != j && phi == s->phase[j])) continue;
            const f3 diff = vsub(pi, s->p[j]);
            const real d2 = vlen2(diff);
            if (d2 <= k->h2 && d2 > 0) eta = vadd(eta, smul(vlen(s->omega[j]), spiky_grad(k, diff, d2)));
        }
        if (vlen2(eta) > 1e-3f) {
            const f3 nn = vnormalize(eta);
            s->v[i] = vadd(s->v[i], vmul(smul(eps, vcross(nn, om)), dt));
        }
    }
}

/* fluidXSph (K/fluid.cuh:338-385) -> out.  Textbook mode weights each
 * neighbour by its volume m_j / rho_j (Macklin & Mueller 2013, eq. 17). */
static void fluid_xsph(or_solver *s, const sph_consts *k, f3 *out)
{
    const real c = s->prm.xsph_c, cell = s->prm.cell_size;
    const int textbook = s->prm.mode == BP_MODE_TEXTBOOK;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < s->n; ++i) {
        const int phi = s->phase[i];
        if (phi >= 0) continue;
        const f3 pi = s->p[i], vi = s->v[i];
        f3 vn = v3(0, 0, 0);
        const i3 c_ = grid_pos(pi, cell);
        FOR_EACH_CANDIDATE(s, pi, j) {
            if (!(i != j && phi == s->phase[j])) continue;
            const real d2 = vlen2(vsub(pi, s->p[j]));
            if (d2 <= k->h2) {
                real wgt = poly6(k, d2);
                if (textbook) wgt = wgt * (s->m[j] / s->rho[j]);
                vn = vadd(vn, vmul(vsub(s->v[j], vi), wgt));
            }
        }
        out[i] = vadd(vi, smul(c, vn));
    }
}

/* fluidNormal (K/fluid.cuh:387-434) */
static void fluid_normal(or_solver *s, const sph_consts *k)
{
    const real cell = s->prm.cell_size;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < s->n; ++i) {
        const int phi = s->phase[i];
        if (phi >= 0) continue;
        const f3 pi = s->p[i];
        f3 nn = v3(0, 0, 0);
        const i3 c_ = grid_pos(pi, cell);
        FOR_EACH_CANDIDATE(s, pi, j) {
            if (!(i != j && phi == s->phase[j])) continue;
            const f3 diff = vsub(pi, s->p[j]);
            const real d2 = vlen2(diff);
            if (d2 <= k->h2 && d2 > 0) nn = vadd(nn, smul(1.0f / s->rho[j], spiky_grad(k, diff, d2)));
        }
        s->normal[i] = smul(k->h, nn);
    }
}

/* fluidAkinciTension (K/fluid.cuh:436-488) -> out (no mass division, Q7) */
static void fluid_akinci(or_solver *s, const sph_consts *k, real dt, f3 *out)
{
    const real g = s->prm.surface_tension, rho0 = s->prm.rest_density, cell = s->prm.cell_size;
#pragma omp parallel for num_threads(g_threads)
    for (int i = 0; i < s->n; ++i) {
        const int phi = s->phase[i];
        if (phi >= 0) continue;
        const f3 pi = s->p[i];
        f3 ft = v3(0, 0, 0);
        const i3 c_ = grid_pos(pi, cell);
        FOR_EACH_CANDIDATE(s, pi, j) {
            if (!(i != j && phi == s->phase[j])) continue;
            const f3 pj = s->p[j];
            const f3 diff = vsub(pi, pj);
            const real d2 = vlen2(diff);
            if (d2 <= k->h2 && d2 > 0.f) {
                const real dist = sqrt(d2);
                const f3 fco = vdiv(smul(-g * akinci_spline(k, dist), vsub(pi, pj)), dist);
                const f3 fcu = smul(-g, vsub(s->normal[i], s->normal[j]));
                const real kij = 2.0f * rho0 / (s->rho[i] + s->rho[j]);
                ft = vadd(ft, smul(kij, vadd(fco, fcu)));
            }
        }
        out[i] = vadd(s->v[i], vmul(ft, dt));
    }
}

static void zero3(f3 *a, int n)
{
    memset(a, 0, sizeof(f3) * (size_t)n);
}

static void acc3(f3 *a, const f3 *d, int n)
{
    for (int i = 0; i < n; ++i) a[i] = vadd(a[i], d[i]);
}

int or_update(or_solver *s, int nsub, float dt, int iterations, int picked, const float *pp, const float *pv)
{
    const int n = s->n;
    if (n <= 0) return 0;
    const bp_params *P = &s->prm;
    const int mask = P->stage_mask;
    const real sdt = dt / (real)nsub;
    const sph_consts k = make_sph(P->kernel_radius, P->mode == BP_MODE_TEXTBOOK);
    const real r = P->particle_radius;
    const f3 g = v3(P->gravity[0], P->gravity[1], P->gravity[2]);
    const f3 ppos = pp ? v3(pp[0], pp[1], pp[2]) : v3(0, 0, 0);
    const f3 pvel = pv ? v3(pv[0], pv[1], pv[2]) : v3(0, 0, 0);
    const int picking = picked >= 0 && picked < n;
    for (int sub = 0; sub < nsub; ++sub) {
        if (picking) { /* PS:790-794 */
            const int id = s->to_new[picked];
            s->x[id] = ppos;
            s->v[id] = v3(0, 0, 0);
        }
        for (int i = 0; i < n; ++i) { /* predictPositions + applyGravity (PS:59-69, 49-57) */
            s->p[i] = vadd(s->x[i], vmul(s->v[i], sdt));
            s->p[i] = vadd(s->p[i], vmul(vmul(g, sdt), sdt));
        }
        update_grid(s);
        for (int i = 0; i < n; ++i) s->to_new[s->to_orig[i]] = i; /* inverseMapping (K/util.cuh:348-358) */
        for (int i = 0; i < n; ++i) { /* computeInvScaledMasses (PS:84-98) */
            const real e = 2.7182818284f;
            const real scale = pow(e, -P->mass_scaling_k * s->x[i].y);
            s->w[i] = 1.0f / (scale * s->m[i]);
        }
        if (mask & BP_STAGE_PLANES)
            for (int it = 0; it < 2; ++it) /* PS:822-833 */
                for (int q = 0; q < s->nplanes; ++q) plane_stabilize(s, plane_o(s, q), plane_n(s, q), r);
        if ((mask & BP_STAGE_WIND) && s->nfaces > 0) { /* PS:838-858 */
            zero3(s->dX, n);
            wind_force(s, sdt);
            acc3(s->p, s->dX, n);
        }
        for (int j = 0; j < iterations; ++j) { /* PS:862-994 */
            if (picking) {
                const int id = s->to_new[picked];
                s->p[id] = ppos;
                s->v[id] = v3(0, 0, 0);
            }
            if (mask & BP_STAGE_PLANES)
                for (int q = 0; q < s->nplanes; ++q) plane_collision(s, plane_o(s, q), plane_n(s, q), r);
            if (mask & BP_STAGE_PARTICLE_COLLISION) {
                zero3(s->dX, n);
                particle_collision(s, r);
                acc3(s->p, s->dX, n);
            }
            if (mask & BP_STAGE_FLUID) {
                memset(s->lambda, 0, sizeof(real) * (size_t)n); /* solids: lambda 0 (Q4) */
                fluid_lambda(s, &k);
                zero3(s->dX, n);
                fluid_position(s, &k);
                acc3(s->p, s->dX, n);
            }
            if ((mask & BP_STAGE_DISTANCE) && s->npairs > 0) {
                zero3(s->dX, n);
                distance_constraints(s);
                acc3(s->p, s->dX, n);
            }
            if ((mask & BP_STAGE_BENDING) && s->nbend > 0) { /* PS:956-969 */
                zero3(s->dX, n);
                bending_constraints(s, s->prm.bending_stiffness);
                acc3(s->p, s->dX, n);
            }
            if ((mask & BP_STAGE_SHAPE_MATCHING) && s->nb > 0) shape_matching(s);
            if ((mask & BP_STAGE_IMMOVABLE) && s->nimm > 0)
                for (int q = 0; q < s->nimm; ++q) { /* immovableConstraints (K/immovable.cuh:3-14) */
                    const int id = s->to_new[s->imm[q]];
                    s->p[id] = s->x[id];
                }
        }
        const real inv_dt = 1.0f / sdt;
        for (int i = 0; i < n; ++i) { /* updateVelocity, updatePositions (PS:71-81, 121-137) */
            s->v[i] = vmul(vsub(s->p[i], s->x[i]), inv_dt);
            s->x[i] = s->p[i];
        }
        if (mask & BP_STAGE_VORTICITY) { /* PS:1004-1022 */
            fluid_omega(s, &k);
            fluid_vorticity(s, &k, sdt);
        }
        if (mask & BP_STAGE_AKINCI) { /* PS:1024-1049: solids keep their velocity (the swap pair cancels) */
            fluid_normal(s, &k);
            memcpy(s->tmp, s->v, sizeof(f3) * (size_t)n);
            fluid_akinci(s, &k, sdt, s->tmp);
            SWAP(s->v, s->tmp);
        }
        if (mask & BP_STAGE_XSPH) { /* PS:1051-1060 */
            memcpy(s->tmp, s->v, sizeof(f3) * (size_t)n);
            fluid_xsph(s, &k, s->tmp);
            SWAP(s->v, s->tmp);
        }
        reset_start_end(n, s->sorted_cell, s->cell_start, s->cell_end); /* PS:1062 */
    }
    if (picking) { /* PS:1065-1071 */
        const int id = s->to_new[picked];
        s->v[id] = pvel;
    }
    return 0;
}

int or_get(or_solver *s, int field, void *out)
{
    const int n = s->n;
    switch (field) {
    case 0: memcpy(out, s->x, sizeof(f3) * (size_t)n); break;
    case 1: memcpy(out, s->p, sizeof(f3) * (size_t)n); break;
    case 2: memcpy(out, s->v, sizeof(f3) * (size_t)n); break;
    case 3: memcpy(out, s->to_orig, sizeof(int) * (size_t)n); break;
    case 4: memcpy(out, s->to_new, sizeof(int) * (size_t)n); break;
    case 5: memcpy(out, s->lambda, sizeof(real) * (size_t)n); break;
    case 6: memcpy(out, s->rho, sizeof(real) * (size_t)n); break;
    case 7: memcpy(out, s->w, sizeof(real) * (size_t)n); break;
    case 8: memcpy(out, s->sorted_cell, sizeof(int) * (size_t)n); break;
    case 9: memcpy(out, s->rot, sizeof(f4) * (size_t)s->nb); break;
    case 10: memcpy(out, s->cms, sizeof(f3) * (size_t)s->nb); break;
    case 11: memcpy(out, s->omega, sizeof(f3) * (size_t)n); break;
    case 12: memcpy(out, s->normal, sizeof(f3) * (size_t)n); break;
    case 13: memcpy(out, s->m, sizeof(real) * (size_t)n); break;
    case 14: memcpy(out, s->phase, sizeof(int) * (size_t)n); break;
    default: return 1;
    }
    return 0;
}
