// bp_common.cuh -- device-side building blocks shared by the solver kernels.
//
// Layout of the particle state in HBM (structure of arrays, cell-sorted):
//   X[i] = float4(x, y, z, mass)            committed position
//   P[i] = float4(px, py, pz, phase bits)   predicted position (the iterate)
//   V[i] = float4(vx, vy, vz, phase bits)   velocity
// plus int32 original ids, a compact float mass array, and per-pass scratch.
// All loads of a particle record are one 16-byte vector load.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/brasspan.h"

namespace bp {

constexpr int kMaxPlanes = 16;

// One scene of a batched ensemble.  The scenes share one key space: scene s
// owns cell keys [base, base + D^3), so one stable sort keeps every scene's
// particles contiguous and in the order a solver of that scene alone gives.
struct SceneConsts {
    int D;             // grid dimension of this scene (power of two)
    unsigned mask;     // D - 1
    int base;          // first cell key of this scene
    int nplanes;
    float rho0, inv_rho0;
    float gx, gy, gz;  // gravity
    float4 plane_o[kMaxPlanes];
    float4 plane_n[kMaxPlanes];
};

// Constants of one substep, passed by value to every kernel (graph friendly).
struct SimConsts {
    int n;
    int D;            // grid dimension (power of two)
    unsigned mask;    // D - 1
    float cell;       // hash cell edge
    // SPH (K/fluid.cuh:11-27), computed on the host with the reference's formulas
    float h, h2, half_h, c_poly6, c_spiky, c_akinci, c_akinci_off;
    // PBF
    float rho0, inv_rho0, solid_scale, lambda_den, relaxation;
    float scorr_k, scorr_inv_wq;       // 1 / poly6((dq*h)^2)
    int scorr_ni;                      // exponent n
    int scorr_on;                      // reference: s_corr only when Akinci is off
    int clamp_c;                       // reference: C = max(C, 0) when Akinci is on
    float delta_clamp, delta_clamp2;   // <= 0: no clamp
    int textbook;
    // post passes
    float vort_eps, tension, xsph_c;
    int use_vort, use_akinci, use_xsph;
    // contacts
    float radius, fs, fd, mass_k;
    float3 gravity;
    float3 wind;
    float wind_drag, wind_lift;
    int rot_iters;
    float dt, inv_dt;
    int nplanes;
    int stage;        // scan kernels stage their neighbourhood in shared memory
    int split;        // scan kernels test candidates in chunks before the pair terms
    int scan_block;   // unstaged scan launches: threads per CTA (bp_params::scan_block; 256 when 0)
    int scan_persist; // unstaged scan launches: at most one resident wave of CTAs, striding over the tiles
    // Contact walks (nullptr: the 27 cells): the bits of floats bounding, per
    // axis, every particle's ([0]) and every solid's ([1]) displacement since
    // its cell was hashed, written by k_contact_reach before the collision
    // pass; the walks then visit only the cells a contact partner can be
    // stored in.
    const unsigned *contact_reach;
    float4 plane_o[kMaxPlanes];
    float4 plane_n[kMaxPlanes];
    // Verlet lists of the current substep (vl == nullptr: off).  The first
    // lambda pass of a substep (vl_build) walks the cells with the radius
    // h + skin and records, for each particle, every candidate within it in
    // walk order (records of four, as SimConsts::nbr; vl_count[i] < 0: did not
    // fit in vl_cap).  nl_cell is the cell the list was built for (-1: the
    // particle always walks its cells, e.g. its column runs wrap around the
    // table), nl_pos its position then.  A later walk of the substep reads the
    // list instead of the cells while the particle is still in nl_cell,
    // within half the skin of nl_pos, and no particle stored in its 27 cells
    // moved further (writers of P flag their stored cell in nl_outlier): then
    // every pair within h now was within h + skin at the build, and the list
    // yields the walk's hits in the walk's order.
    int *vl;
    int *vl_count;
    int vl_cap;
    int vl_build;                      // this launch builds the lists
    int *nl_cell;
    float4 *nl_pos;                    // nullptr: writers do not track displacements
    unsigned long long *nl_outlier;    // per (x, y) column of cells, nl_zwords words of z bits
    int nl_zwords;                     // ceil(D / 64)
    const int *cell_keys;              // stored cell of every sorted particle
    unsigned *nl_stats;      // profiling only: walks by list_state, then alias-class walks
    float nl_hs2;            // (h + skin)^2
    float nl_half_skin2;     // (skin / 2)^2
    // Neighbour lists, written by one pass and read by the following ones at
    // the same positions: by lambda for the position pass (every j with
    // r^2 <= h^2), by post pass A for passes B and C (same-phase j != i).
    // Entry k of particle i is nbr[((k / 4) * n + i) * 4 + k % 4], in walk
    // order, for k < nbr_count[i]: each group of four is one 16-byte record,
    // so a warp writes and reads whole records.  nbr_count[i] < 0 when they
    // did not fit in nbr_cap entries (a multiple of 4; the readers then walk
    // the cells).
    int *nbr;
    int *nbr_count;
    int nbr_cap;
    // With the position pass's lists: (lambda, mass) of every sorted particle,
    // written by k_lambda beside lam where its lists hold sorted indices.
    float2 *lm;
    // Batched ensembles (nullptr: one scene, described by the fields above).
    // scene_of[i] is the scene of particle i; it holds for sorted and
    // original indices alike, because every scene keeps its segment.
    const SceneConsts *scn;
    const int *scene_of;
    // Alias classes (cls_perm == nullptr: off).  A table of D^3 cells wraps
    // space: table cell (x, y, z) holds the particles of every real cell
    // (x + aD, y + bD, z + cD).  At hash time each particle gets the parity
    // bits of (a, b, c), its class (0..7).  cls_perm lists the sorted indices
    // class by class, each class in ascending sorted index, cls_inv is its
    // inverse and cls_off[k * cls_T + key] the dense prefix over (class, cell
    // key).  A walk of real cell w visits only the particles of w's class in
    // that table cell: any other one was hashed at least D - 2 cells from the
    // walker along some axis, so it fails every distance test within h while
    // no particle has moved further than the reach (D - 2) cell - h - margin
    // from its hash-time position.  k_class_refresh gathers P into cls_pos
    // before each walking launch and sets *cls_moved when some particle moved
    // further; walks then take whole table cells for the rest of the substep.
    const int *cls_perm;
    const int *cls_inv;
    const int *cls_of;      // class of each sorted particle
    const int *cls_off;     // [8 * cls_T + 1]
    const float4 *cls_pos;  // P in class order
    const int *cls_moved;
    int cls_T;              // cell keys of all scenes
    // Class-order copies for the position pass's slot lists (k_lambda):
    // masses (k_class_keys) and (lambda, mass) pairs k_lambda writes beside
    // lam, which the position pass gathers in one 8-byte load per neighbour.
    const float *cls_mass;
    float2 *cls_lm;
    // And for the post passes' slot lists (k_post_a), used where cls_post is
    // set (a lambda pass of the substep wrote cls_rho): densities, committed
    // velocities (gathered with the positions before pass A), pass A's
    // vorticities and normals, pass B's velocities.
    float *cls_rho;
    float4 *cls_vel, *cls_om, *cls_nm, *cls_vb;
    int cls_post;
    // Walk planes (nullptr: off): x, y, z and the phase bits of every
    // particle in four planes of walk_stride floats (a multiple of 4, at
    // least n + kPlanePad), written just before the lambda pass and post
    // pass A, whose recording walks test four candidates per three 16-byte
    // loads with paired fp32 arithmetic and append each chunk's hits to the
    // list a record at a time.  They hold class order while the classes are
    // on and sorted order where the classes are closed or absent (see
    // walk_planes_order).
    const float *walk_xyz;
    int walk_stride;
};

// The walks use the alias classes for the rest of the substep (uniform
// over a launch: the flag is written by k_class_refresh before it).
// *cls_moved: 0 classes on, 1 gate closed, 2 a particle left the reach.
__device__ __forceinline__ bool classes_on(const SimConsts &C)
{
    return C.cls_perm && __ldg(C.cls_moved) == 0;
}

// Quads of candidates a recording walk over the walk planes tests per loop
// trip (loads in flight: three per quad).
#ifndef BP_PLANE_QUADS
#define BP_PLANE_QUADS 1
#endif
constexpr int kPlaneQuads = BP_PLANE_QUADS;
// Floats past n a walk-plane read may reach: the last trip of a chunk reads
// up to kPlaneQuads quads from an aligned start below the run's end.
constexpr int kPlanePad = 4 * kPlaneQuads + 4;

// Order of the walk planes: 2 class order (the classes are on), 1 sorted
// order (no classes, or their gate is closed: k_class_refresh then writes
// the planes in sorted order), 0 none usable (no planes, or the classes
// closed because a particle left the reach after the planes were written in
// class order).
__device__ __forceinline__ int walk_planes_order(const SimConsts &C)
{
    if (!C.walk_xyz) return 0;
    if (!C.cls_perm) return 1;
    const int m = __ldg(C.cls_moved);
    return m == 0 ? 2 : (m == 1 ? 1 : 0);
}

// Class (0..7) of real cell c on a table of D cells per axis (D a power of two).
__device__ __forceinline__ int alias_class(int x, int y, int z, int D)
{
    const int sh = __ffs(D) - 1;
    return ((x >> sh) & 1) | (((y >> sh) & 1) << 1) | (((z >> sh) & 1) << 2);
}

// ---- small vector helpers (own code) ----
// Every operation is an explicitly rounded intrinsic, so the compiler never
// fuses or reorders arithmetic differently in two inlined copies of the same
// expression: a pair term evaluates to the same bits wherever it is used.

__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b)
{
    return make_float3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z));
}
__device__ __forceinline__ float3 operator-(float3 a, float3 b)
{
    return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s)
{
    return make_float3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s));
}
__device__ __forceinline__ float3 operator*(float s, float3 a) { return a * s; }
__device__ __forceinline__ float3 operator/(float3 a, float s)
{
    return make_float3(__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s));
}
__device__ __forceinline__ void operator+=(float3 &a, float3 b) { a = a + b; }
__device__ __forceinline__ void operator-=(float3 &a, float3 b) { a = a - b; }
// a + s * b with one rounding per component
__device__ __forceinline__ float3 fma3(float s, float3 b, float3 a)
{
    return make_float3(__fmaf_rn(s, b.x, a.x), __fmaf_rn(s, b.y, a.y), __fmaf_rn(s, b.z, a.z));
}
__device__ __forceinline__ float dot3(float3 a, float3 b)
{
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return make_float3(__fmaf_rn(a.y, b.z, -__fmul_rn(a.z, b.y)), __fmaf_rn(a.z, b.x, -__fmul_rn(a.x, b.z)),
                       __fmaf_rn(a.x, b.y, -__fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float len2(float3 a) { return dot3(a, a); }
__device__ __forceinline__ float len3(float3 a) { return __fsqrt_rn(dot3(a, a)); }
__device__ __forceinline__ int phase_of(float4 a) { return __float_as_int(a.w); }

// ---- SPH kernels (same formulas as K/fluid.cuh:31-74) ----

__device__ __forceinline__ float poly6(const SimConsts &C, float r2)
{
    const float t = __fsub_rn(C.h2, r2);
    return __fmul_rn(__fmul_rn(__fmul_rn(C.c_poly6, t), t), t);
}
__device__ __forceinline__ float3 spiky_grad(const SimConsts &C, float3 v, float r2)
{
    const float r = __fsqrt_rn(r2);
    const float t = __fsub_rn(C.h, r);
    return (__fmul_rn(__fmul_rn(C.c_spiky, t), t) * v) / r;
}
// Same gradient through one reciprocal square root (r2 > 0): the hot loops'
// form.  Differs from the IEEE sqrt-and-divide form above by a few ulp.
__device__ __forceinline__ float3 spiky_grad_r(const SimConsts &C, float3 v, float r2, float inv_r)
{
    const float t = __fmaf_rn(-r2, inv_r, C.h);
    return __fmul_rn(__fmul_rn(__fmul_rn(C.c_spiky, t), t), inv_r) * v;
}
__device__ __forceinline__ float ipowf(float x, int n)
{
    float r = 1.0f;
    for (int k = 0; k < n; ++k) r = __fmul_rn(r, x);
    return r;
}
__device__ __forceinline__ float akinci_spline(const SimConsts &C, float r)
{
    const float t = __fmul_rn(__fsub_rn(C.h, r), r);
    const float t3 = __fmul_rn(__fmul_rn(t, t), t);
    return (r >= C.half_h) ? __fmul_rn(C.c_akinci, t3)
                           : __fsub_rn(__fmul_rn(__fmul_rn(2.0f, C.c_akinci), t3), C.c_akinci_off);
}

// ---- hash grid (same cell function as K/grid.cuh:9-28) ----
// cell = trunc((p + 50000) / cell) with IEEE add and divide.

__device__ __forceinline__ int cell_coord(float p, float cell)
{
    return (int)__fdiv_rn(__fadd_rn(p, 50000.0f), cell);
}
__device__ __forceinline__ int3 cell_of(float3 p, const SimConsts &C)
{
    return make_int3(cell_coord(p.x, C.cell), cell_coord(p.y, C.cell), cell_coord(p.z, C.cell));
}
__device__ __forceinline__ int cell_addr(int x, int y, int z, int D, unsigned mask)
{
    return (int)(((unsigned)x & mask) * ((unsigned)D * (unsigned)D) + ((unsigned)y & mask) * (unsigned)D +
                 ((unsigned)z & mask));
}

// The grid a particle's walks use: its scene's dimension, and the cell
// offsets from its scene's first key on (off[0] is that scene's first cell).
struct GridView {
    int D;
    unsigned mask;
    int base;
    const int *off;
};
__device__ __forceinline__ int scene_index(const SimConsts &C, int i)
{
    return C.scene_of ? __ldg(C.scene_of + i) : -1;
}
__device__ __forceinline__ GridView grid_view(const SimConsts &C, int s, const int *off)
{
    if (s < 0) return GridView{C.D, C.mask, 0, off};
    const SceneConsts &S = C.scn[s];
    const int base = S.base;
    return GridView{S.D, S.mask, base, off + base};
}
__device__ __forceinline__ float rest_density(const SimConsts &C, int s) { return s < 0 ? C.rho0 : C.scn[s].rho0; }
__device__ __forceinline__ float inv_rest_density(const SimConsts &C, int s)
{
    return s < 0 ? C.inv_rho0 : C.scn[s].inv_rho0;
}
__device__ __forceinline__ float3 gravity_of(const SimConsts &C, int s)
{
    return s < 0 ? C.gravity : make_float3(C.scn[s].gx, C.scn[s].gy, C.scn[s].gz);
}

// Is any of the cells (x, y, z0..z0+2) flagged as holding an outlier (a
// particle that moved more than half the skin since the lists were built)?
// z0 + 2 < D: lists are only built where the column runs do not wrap.
__device__ __forceinline__ bool column_has_outlier(const SimConsts &C, unsigned x, unsigned y, unsigned z0)
{
    const unsigned long long *w = C.nl_outlier + (size_t)(x * (unsigned)C.D + y) * C.nl_zwords;
    const unsigned k = z0 >> 6, s = z0 & 63u;
    // flags written by earlier kernels; a flag set during this kernel concerns
    // positions this kernel does not read, so a stale read is harmless
    unsigned long long bits = __ldg(w + k) >> s;
    if (s > 61u && k + 1 < (unsigned)C.nl_zwords) bits |= __ldg(w + k + 1) << (64u - s);
    return (bits & 7ull) != 0ull;
}

// 0 when particle i may read its Verlet list instead of walking its 27
// cells; otherwise why not: 1 no list for it, 2 it changed cell, 3 it, or a
// particle stored in its 27 cells, moved more than half the skin since the build.
__device__ __forceinline__ int list_state(const SimConsts &C, int i, int3 c, float3 pi)
{
    const int built = __ldg(C.nl_cell + i);
    if (built < 0) return 1;
    if (built != cell_addr(c.x, c.y, c.z, C.D, C.mask)) return 2;
    if (len2(pi - f3(C.nl_pos[i])) > C.nl_half_skin2) return 3;
    const unsigned m = C.mask;
    const unsigned z0 = (unsigned)(c.z - 1) & m;
    for (int col = 0; col < 9; ++col)
        if (column_has_outlier(C, (unsigned)(c.x + col / 3 - 1) & m, (unsigned)(c.y + col % 3 - 1) & m, z0))
            return 3;
    return 0;
}

// Records that particle i moved more than half the skin since the list
// build: flags its stored cell (the cell its sorted index belongs to) so the
// particles whose 27 cells include it walk their cells.  Writers of P call it
// with the new position.
__device__ __forceinline__ void track_displacement(const SimConsts &C, int i, float3 p, bool active)
{
    if (!C.nl_pos || !active) return;
    if (!(len2(p - f3(C.nl_pos[i])) <= C.nl_half_skin2)) {  // NaN counts as moved
        const unsigned key = (unsigned)__ldg(C.cell_keys + i);
        const unsigned col = key / (unsigned)C.D, z = key % (unsigned)C.D;
        atomicOr(C.nl_outlier + (size_t)col * C.nl_zwords + (z >> 6), 1ull << (z & 63u));
    }
}

// Plane walls: planeStabilize / particlePlaneCollisionConstraint
// (K/particleplane.cuh:3-58) for one particle, planes in scene order.
// In a batched ensemble, scene s uses its own planes (s >= 0).
template <class Planes>
__device__ __forceinline__ void plane_stabilize_with(const SimConsts &C, int np, Planes planes, float3 &x, float3 &p)
{
    for (int k = 0; k < np; ++k) {
        float3 o, nn;
        planes(k, o, nn);
        const float d = dot3(o - x, nn) + C.radius;
        if (d <= 0.f) continue;
        x += d * nn;
        p += d * nn;
    }
}
template <class Planes>
__device__ __forceinline__ void plane_collide_with(const SimConsts &C, int np, Planes planes, float3 x, float3 &p)
{
    for (int k = 0; k < np; ++k) {
        float3 o, nn;
        planes(k, o, nn);
        const float d = dot3(o - p, nn) + C.radius;
        if (d <= 0.f) continue;
        const float3 diff = p - x;
        const float dn = dot3(diff, nn);
        const float3 dt = diff - dn * nn;
        const float dtl = len3(dt);
        const float3 resolved = d * nn + p;
        const float3 dx = resolved - x;
        const float3 tdx = dx - dot3(dx, nn) * nn;
        if (dtl < C.fs * dn)
            p = resolved - tdx;
        else
            p = resolved - tdx * fminf(C.fd * -dn / dtl, 1.0f);
    }
}
// Planes of scene s (s < 0: the solver's one scene).
__device__ __forceinline__ void plane_stabilize(const SimConsts &C, int s, float3 &x, float3 &p)
{
    if (s < 0) {
        plane_stabilize_with(
            C, C.nplanes, [&](int k, float3 &o, float3 &n) { o = f3(C.plane_o[k]); n = f3(C.plane_n[k]); }, x, p);
    } else {
        const SceneConsts &S = C.scn[s];
        plane_stabilize_with(
            C, S.nplanes, [&](int k, float3 &o, float3 &n) { o = f3(S.plane_o[k]); n = f3(S.plane_n[k]); }, x, p);
    }
}
__device__ __forceinline__ void plane_collide(const SimConsts &C, int s, float3 x, float3 &p)
{
    if (s < 0) {
        plane_collide_with(
            C, C.nplanes, [&](int k, float3 &o, float3 &n) { o = f3(C.plane_o[k]); n = f3(C.plane_n[k]); }, x, p);
    } else {
        const SceneConsts &S = C.scn[s];
        plane_collide_with(
            C, S.nplanes, [&](int k, float3 &o, float3 &n) { o = f3(S.plane_o[k]); n = f3(S.plane_n[k]); }, x, p);
    }
}

}  // namespace bp
