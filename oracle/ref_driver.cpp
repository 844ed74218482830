/*
 * ref_driver.cpp -- runs brass-pan's OWN kernel bodies on the host.
 *
 * TEST INFRASTRUCTURE (the reference build, "oracle/_ref"): this file is
 * compiled together with the reference's unmodified kernel headers
 * (brasstower/kernel/{grid,fluid,particleplane,particleparticle,distance,wind,
 * shapematching,immovable,bending}.cuh, cuda/cudamatrix.cuh, ext/helper_math.h), read
 * in place from the reference checkout through the host shim in
 * oracle/refshim/.  Its outputs pin the C restatement (oracle/oracle.c) and
 * are committed as golden fixtures under tests/golden/.  Nothing in the
 * product links or calls it.
 *
 * What is ours here: the launch emulation (an OpenMP loop over the flattened
 * thread index; shapeMatchingAlphaOne runs each 64-thread block as an OpenMP
 * team), a stable std::stable_sort standing in for cub::DeviceRadixSort
 * (identical result: LSD radix sort is stable), and the replay of
 * ParticleSolver::update() (particlesolver.cuh:772-1072) with the commented
 * constraint block (:881-993) and wind block (:838-858) enabled and the
 * solver-iteration count and the mass-scaling k as parameters.  The few
 * one-line kernels defined inside particlesolver.cuh (which cannot be parsed
 * by a host compiler: it uses <<<>>> launches, conio.h and MSVC-only
 * exceptions) are restated below with their line numbers.
 *
 * Defined behaviour where the reference reads uninitialised memory: the lambda
 * of a solid particle (fluid.cuh:207 reads lambdas[j] that fluidLambda never
 * wrote for solids) is 0, because the lambda buffer is zeroed before every
 * fluidLambda launch.
 */
#include <omp.h>
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <numeric>
#include <vector>

#include "cuda_runtime.h" /* refshim */

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

#include "kernel/grid.cuh"
#include "kernel/fluid.cuh"

#include "kernel/particleplane.cuh"
#include "kernel/particleparticle.cuh"
#include "kernel/distance.cuh"
#include "kernel/wind.cuh"
#include "kernel/shapematching.cuh"
#include "kernel/immovable.cuh"

/* kernel/bending.cuh:52 negates a temporary, which helper_math.h's
 * operator-(float3 &) cannot bind; this overload for rvalues (ours) lets the
 * unmodified kernel compile. */
inline __host__ __device__ float3 operator-(float3 &&a) { return make_float3(-a.x, -a.y, -a.z); }
#include "kernel/bending.cuh"

#include "../include/brasspan.h"

static int g_threads = 1;

/* Launch emulation: one loop iteration per CUDA thread, 128-thread blocks as
 * GetNumBlocksNumThreads (kernel/util.cuh:3-8). */
template <class F>
static void launch(int count, F &&body)
{
    if (count <= 0) return;
    const int threads = 128;
    const int blocks = (count + threads - 1) / threads;
    const long total = (long)blocks * threads;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (long g = 0; g < total; ++g) {
        blockIdx = make_uint3((unsigned)(g / threads), 0, 0);
        threadIdx = make_uint3((unsigned)(g % threads), 0, 0);
        blockDim = dim3(threads, 1, 1);
        body();
    }
}

/* ---- one-line kernels of particlesolver.cuh, restated ------------------- */

static void k_applyGravity(float3 *p, int n, float dt) /* particlesolver.cuh:49-57 */
{
    launch(n, [&] {
        int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
        if (i >= n) return;
        p[i] += make_float3(0.0f, -9.8f, 0.0f) * dt * dt;
    });
}

static void k_predictPositions(float3 *np, const float3 *x, const float3 *v, int n, float dt) /* :59-69 */
{
    launch(n, [&] {
        int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
        if (i >= n) return;
        np[i] = x[i] + v[i] * dt;
    });
}

static void k_updateVelocity(float3 *v, const float3 *np, const float3 *x, int n, float invDt) /* :71-81 */
{
    launch(n, [&] {
        int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
        if (i >= n) return;
        v[i] = (np[i] - x[i]) * invDt;
    });
}

static void k_computeInvScaledMasses(float *w, const float *m, const float3 *x, float k, int n) /* :84-98 */
{
    launch(n, [&] {
        int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
        if (i >= n) return;
        const float e = 2.7182818284f;
        const float height = x[i].y;
        const float scale = pow(e, -k * height);
        w[i] = 1.0f / (scale * m[i]);
    });
}

static void k_updatePositions(float3 *x, const float3 *np, const int *phases, float thr, int n) /* :121-137 */
{
    launch(n, [&] {
        int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
        if (i >= n) return;
        const float3 xi = x[i];
        const float3 nx = np[i];
        const float d2 = length2(nx - xi);
        x[i] = (d2 >= thr * thr || phases[i] < 0) ? nx : xi;
    });
}

static void k_inverseMapping(int *toNew, const int *toOrig, int n) /* kernel/util.cuh:348-358 */
{
    launch(n, [&] {
        int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
        if (i >= n) return;
        toNew[toOrig[i]] = i;
    });
}

template <class T>
static void k_fill(T *a, T v, int n)
{
    launch(n, [&] {
        int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
        if (i >= n) return;
        a[i] = v;
    });
}

static void k_acc(float3 *a, const float3 *d, int n) /* accDevArr_float3, kernel/util.cuh:261-269 */
{
    launch(n, [&] {
        int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
        if (i >= n) return;
        a[i] += d[i];
    });
}

/* ---- the solver state, mirroring ParticleSolver's device arrays --------- */

struct RefSolver {
    int n = 0;
    float radius = 0, h = 0, cell = 0, restDensity = 0;
    float massScalingK = 2.0f; /* MASS_SCALING_CONSTANT (cubrasstower.cuh:20), passed at :809 */
    int D = 0;
    std::vector<float3> x, p, v, sx, sp, sv, dX, tmp, omegas, normals;
    std::vector<float> m, sm, invScaled, lambdas, densities;
    std::vector<int> phase, sphase, group, sgroup, toOrig, stoOrig, toNew;
    std::vector<int> cellId, particleId, sortedCellId, sortedParticleId, cellStart, cellEnd;
    std::vector<int2> ranges, pairs;
    std::vector<float2> dparams;
    std::vector<float3> rest;
    std::vector<float4> rotations;
    std::vector<float3> cms;
    std::vector<int3> faces;
    std::vector<int> immovables;
    std::vector<int4> bends;
    std::vector<float3> planeO, planeN;
};

static void set_constants(const RefSolver &s)
{
    SetKernelRadius(s.h); /* fluid.cuh:11-27, the reference's own host code */
    GridDim = (uint)s.D;
    GridCellSize = make_float3(s.cell);
}

/* updateGrid (particlesolver.cuh:712-765) */
static void update_grid(RefSolver &s)
{
    const int n = s.n;
    int *cid = s.cellId.data(), *pid = s.particleId.data();
    const float3 *np = s.p.data();
    float3 cellOrigin = make_float3(0.f);
    int3 gridSize = make_int3(s.D);
    float3 cs = make_float3(s.cell);
    launch(n, [&] { updateGridId(cid, pid, np, cellOrigin, cs, gridSize, n); });
    /* cub::DeviceRadixSort::SortPairs: stable by key */
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cid[a] < cid[b]; });
    for (int i = 0; i < n; ++i) {
        s.sortedCellId[i] = cid[order[i]];
        s.sortedParticleId[i] = pid[order[i]];
    }
    int *cst = s.cellStart.data(), *cen = s.cellEnd.data();
    const int *scid = s.sortedCellId.data();
    launch(n, [&] { findStartEndId(cst, cen, scid, n); });
    float3 *snp = s.sp.data(), *sx = s.sx.data(), *sv = s.sv.data();
    float *sm = s.sm.data();
    int *sph = s.sphase.data(), *sto = s.stoOrig.data(), *sg = s.sgroup.data();
    const float3 *x = s.x.data(), *v = s.v.data();
    const float *m = s.m.data();
    const int *ph = s.phase.data(), *g = s.group.data(), *to = s.toOrig.data(),
              *spid = s.sortedParticleId.data();
    launch(n, [&] {
        reorderParticlesData(snp, sx, sv, sm, sph, sto, sg, np, x, v, m, ph, g, to, spid, n);
    });
    std::swap(s.sp, s.p);
    std::swap(s.sx, s.x);
    std::swap(s.sv, s.v);
    std::swap(s.sm, s.m);
    std::swap(s.sphase, s.phase);
    std::swap(s.sgroup, s.group);
    std::swap(s.stoOrig, s.toOrig);
}

static void set_particle(RefSolver &s, std::vector<float3> &pos, int idx, float3 p, float3 vel)
{ /* setParticle (particlesolver.cuh:388-393) */
    if (idx < 0 || idx >= s.n) return;
    pos[idx] = p;
    s.v[idx] = vel;
}

static void update(RefSolver &s, int numSub, float dt, int iterations, int mask, int picked,
                   float3 pickedPos, float3 pickedVel)
{
    if (s.n <= 0) return;
    set_constants(s);
    const int n = s.n;
    const float subDt = dt / (float)numSub;
    const bool useAkinci = (mask & BP_STAGE_AKINCI) != 0; /* hard-coded true (:785) */
    for (int sub = 0; sub < numSub; ++sub) {
        if (picked >= 0 && picked < n) set_particle(s, s.x, s.toNew[picked], pickedPos, make_float3(0.f));

        k_predictPositions(s.p.data(), s.x.data(), s.v.data(), n, subDt);
        k_applyGravity(s.p.data(), n, subDt);
        update_grid(s);
        k_inverseMapping(s.toNew.data(), s.toOrig.data(), n);
        k_computeInvScaledMasses(s.invScaled.data(), s.m.data(), s.x.data(), s.massScalingK, n);

        float3 *x = s.x.data(), *p = s.p.data(), *v = s.v.data(), *dX = s.dX.data();
        const int *cst = s.cellStart.data(), *cen = s.cellEnd.data(), *ph = s.phase.data();
        const float *m = s.m.data(), *w = s.invScaled.data();
        const int *toNew = s.toNew.data();
        const float r = s.radius;

        if (mask & BP_STAGE_PLANES)
            for (int it = 0; it < 2; ++it) /* :822-833 */
                for (size_t k = 0; k < s.planeO.size(); ++k) {
                    float3 o = s.planeO[k], nn = s.planeN[k];
                    launch(n, [&] { planeStabilize(x, p, n, o, nn, r); });
                }

        if ((mask & BP_STAGE_WIND) && !s.faces.empty()) { /* :838-858 */
            k_fill(dX, make_float3(0.f), n);
            const int nf = (int)s.faces.size();
            const int3 *f = s.faces.data();
            launch(nf, [&] { applyWindForce(dX, p, v, m, toNew, f, nf, subDt); });
            k_acc(p, dX, n);
        }

        for (int j = 0; j < iterations; ++j) { /* :862-994 */
            if (picked >= 0 && picked < n) set_particle(s, s.p, s.toNew[picked], pickedPos, make_float3(0.f));
            if (mask & BP_STAGE_PLANES)
                for (size_t k = 0; k < s.planeO.size(); ++k) {
                    float3 o = s.planeO[k], nn = s.planeN[k];
                    launch(n, [&] { particlePlaneCollisionConstraint(p, x, n, o, nn, r); });
                }
            if (mask & BP_STAGE_PARTICLE_COLLISION) {
                k_fill(dX, make_float3(0.f), n);
                launch(n, [&] { particleParticleCollisionConstraint(dX, p, x, w, ph, cst, cen, n, r); });
                k_acc(p, dX, n);
            }
            if (mask & BP_STAGE_FLUID) {
                float *lam = s.lambdas.data(), *rho = s.densities.data();
                k_fill(lam, 0.0f, n); /* defined lambda for solids, see header */
                const float rd = s.restDensity;
                launch(n, [&] { fluidLambda(lam, rho, p, m, ph, rd, 2.0f, 300.0f, cst, cen, n, useAkinci); });
                k_fill(dX, make_float3(0.f), n);
                launch(n, [&] { fluidPosition(dX, p, lam, rd, m, ph, 0.0001f, 4, cst, cen, n, useAkinci); });
                k_acc(p, dX, n);
            }
            if ((mask & BP_STAGE_DISTANCE) && !s.pairs.empty()) {
                k_fill(dX, make_float3(0.f), n);
                const int np_ = (int)s.pairs.size();
                const int2 *pr = s.pairs.data();
                const float2 *pa = s.dparams.data();
                launch(np_, [&] { distanceConstraints(dX, p, w, pr, pa, toNew, np_); });
                k_acc(p, dX, n);
            }
            if ((mask & BP_STAGE_BENDING) && !s.bends.empty()) { /* PS:956-969 */
                k_fill(dX, make_float3(0.f), n);
                const int nq = (int)s.bends.size();
                const int4 *bq = s.bends.data();
                launch(nq, [&] { bendingConstraints(dX, p, w, bq, toNew, nq); });
                k_acc(p, dX, n);
            }
            if ((mask & BP_STAGE_SHAPE_MATCHING) && !s.ranges.empty()) {
                const int nb = (int)s.ranges.size();
                float4 *rot = s.rotations.data();
                float3 *cms = s.cms.data();
                const float3 *rest = s.rest.data();
                const int2 *rg = s.ranges.data();
                for (int b = 0; b < nb; ++b) {
#pragma omp parallel num_threads(NUM_MAX_PARTICLE_PER_RIGID_BODY)
                    {
                        blockIdx = make_uint3(b, 0, 0);
                        threadIdx = make_uint3(omp_get_thread_num(), 0, 0);
                        blockDim = dim3(NUM_MAX_PARTICLE_PER_RIGID_BODY, 1, 1);
                        shapeMatchingAlphaOne(rot, cms, p, toNew, rest, rg);
                    }
                }
            }
            if ((mask & BP_STAGE_IMMOVABLE) && !s.immovables.empty()) {
                const int ni = (int)s.immovables.size();
                const int *im = s.immovables.data();
                launch(ni, [&] { immovableConstraints(p, x, im, toNew, ni); });
            }
        }

        k_updateVelocity(v, p, x, n, 1.0f / subDt);
        k_updatePositions(x, p, ph, 0.0f, n);

        {
            const int *cst2 = cst, *cen2 = cen;
            float3 *om = s.omegas.data(), *nm = s.normals.data(), *tmp = s.tmp.data();
            const float *rho = s.densities.data();
            const float rd = s.restDensity;
            if (mask & BP_STAGE_VORTICITY) {
                launch(n, [&] { fluidOmega(om, v, p, ph, cst2, cen2, n); });
                launch(n, [&] { fluidVorticity(v, om, p, 0.001f, ph, cst2, cen2, n, subDt); });
            }
            if (useAkinci) {
                launch(n, [&] { fluidNormal(nm, p, rho, ph, cst2, cen2, n); });
                launch(n, [&] { fluidAkinciTension(tmp, v, p, nm, rho, rd, ph, 0.5f, cst2, cen2, n, subDt); });
                std::swap(s.v, s.tmp);
                v = s.v.data();
                tmp = s.tmp.data();
            }
            if (mask & BP_STAGE_XSPH) {
                launch(n, [&] { fluidXSph(tmp, v, p, 0.0002f, ph, cst2, cen2, n); });
                std::swap(s.v, s.tmp);
            }
        }
        {
            int *cst3 = s.cellStart.data(), *cen3 = s.cellEnd.data();
            const int *scid = s.sortedCellId.data();
            launch(n, [&] { resetStartEndId(cst3, cen3, scid, n); });
        }
    }
    if (picked >= 0 && picked < n) {
        int id = s.toNew[picked];
        set_particle(s, s.x, id, s.x[id], pickedVel);
    }
}

/* ---- C ABI for the Python test harness ---------------------------------- */

extern "C" {

void ref_set_threads(int t) { g_threads = t > 0 ? t : 1; }

void *ref_create(const bp_scene_desc *sc, float radius, float h, float cell, int D, float restDensity)
{
    RefSolver *s = new RefSolver();
    const int n = sc->num_particles;
    s->n = n;
    s->radius = radius;
    s->h = h;
    s->cell = cell;
    s->D = D;
    s->restDensity = restDensity;
    auto f3 = [](const float *a, int i) { return make_float3(a[3 * i], a[3 * i + 1], a[3 * i + 2]); };
    s->x.resize(n); s->p.resize(n); s->v.resize(n); s->sx.resize(n); s->sp.resize(n); s->sv.resize(n);
    s->dX.resize(n); s->tmp.resize(n); s->omegas.resize(n); s->normals.resize(n);
    s->m.resize(n); s->sm.resize(n); s->invScaled.resize(n); s->lambdas.assign(n, 0.f); s->densities.assign(n, 0.f);
    s->phase.resize(n); s->sphase.resize(n); s->group.assign(n, 0); s->sgroup.assign(n, 0);
    s->toOrig.resize(n); s->stoOrig.resize(n);
    s->toNew.assign(n + 64, 0); /* shapeMatchingAlphaOne reads newIds past a body's end */
    for (int i = 0; i < n; ++i) {
        s->x[i] = f3(sc->positions, i);
        s->p[i] = s->x[i];
        s->v[i] = sc->velocities ? f3(sc->velocities, i) : make_float3(0.f);
        s->m[i] = sc->masses[i];
        s->phase[i] = sc->phases[i];
        if (sc->group_ids) s->group[i] = sc->group_ids[i];
        s->toOrig[i] = i;
        s->toNew[i] = i;
    }
    s->cellId.resize(n); s->particleId.resize(n); s->sortedCellId.resize(n); s->sortedParticleId.resize(n);
    size_t cells = (size_t)D * D * D;
    s->cellStart.assign(cells, -1);
    s->cellEnd.assign(cells, -1);
    for (int k = 0; k < sc->num_planes; ++k) {
        s->planeO.push_back(f3(sc->planes + 6 * k, 0));
        s->planeN.push_back(f3(sc->planes + 6 * k + 3, 0));
    }
    for (int k = 0; k < sc->num_distance_constraints; ++k) {
        s->pairs.push_back(make_int2(sc->distance_pairs[2 * k], sc->distance_pairs[2 * k + 1]));
        s->dparams.push_back(make_float2(sc->distance_params[2 * k], sc->distance_params[2 * k + 1]));
    }
    for (int k = 0; k < sc->num_wind_faces; ++k)
        s->faces.push_back(make_int3(sc->wind_faces[3 * k], sc->wind_faces[3 * k + 1], sc->wind_faces[3 * k + 2]));
    for (int k = 0; k < sc->num_rigid_bodies; ++k)
        s->ranges.push_back(make_int2(sc->rigid_ranges[2 * k], sc->rigid_ranges[2 * k + 1]));
    s->rest.assign(n + 64, make_float3(0.f));
    if (sc->rigid_rest_positions)
        for (int i = 0; i < n; ++i) s->rest[i] = f3(sc->rigid_rest_positions, i);
    s->rotations.assign(s->ranges.size(), make_float4(0.f, 0.f, 0.f, 1.f));
    s->cms.assign(s->ranges.size(), make_float3(0.f));
    for (int k = 0; k < sc->num_immovables; ++k) s->immovables.push_back(sc->immovables[k]);
    for (int k = 0; k < sc->num_bendings; ++k)
        s->bends.push_back(make_int4(sc->bendings[4 * k], sc->bendings[4 * k + 1], sc->bendings[4 * k + 2],
                                     sc->bendings[4 * k + 3]));
    return s;
}

void ref_destroy(void *h) { delete (RefSolver *)h; }

/* The k of the inverse scaled masses (the literal MASS_SCALING_CONSTANT = 2
 * at the reference's call site) as a parameter. */
void ref_set_mass_scaling(void *h, float k) { ((RefSolver *)h)->massScalingK = k; }

int ref_update(void *h, int numSub, float dt, int iterations, int mask, int picked, const float *pp,
               const float *pv)
{
    RefSolver *s = (RefSolver *)h;
    float3 p = pp ? make_float3(pp[0], pp[1], pp[2]) : make_float3(0.f);
    float3 v = pv ? make_float3(pv[0], pv[1], pv[2]) : make_float3(0.f);
    update(*s, numSub, dt, iterations, mask, picked, p, v);
    return 0;
}

/* field ids: 0 x, 1 p, 2 v (float3 [N]); 3 toOrig, 4 toNew (int [N]); 5 lambdas, 6 densities,
 * 7 invScaled (float [N]); 8 sortedCellId (int [N]); 9 rotations (float4 [B]); 10 cms (float3 [B]);
 * 11 omegas, 12 normals (float3 [N]); 13 mass (float [N]); 14 phase (int [N]) */
int ref_get(void *h, int field, void *out)
{
    RefSolver *s = (RefSolver *)h;
    const int n = s->n;
    switch (field) {
    case 0: memcpy(out, s->x.data(), n * sizeof(float3)); break;
    case 1: memcpy(out, s->p.data(), n * sizeof(float3)); break;
    case 2: memcpy(out, s->v.data(), n * sizeof(float3)); break;
    case 3: memcpy(out, s->toOrig.data(), n * sizeof(int)); break;
    case 4: memcpy(out, s->toNew.data(), n * sizeof(int)); break;
    case 5: memcpy(out, s->lambdas.data(), n * sizeof(float)); break;
    case 6: memcpy(out, s->densities.data(), n * sizeof(float)); break;
    case 7: memcpy(out, s->invScaled.data(), n * sizeof(float)); break;
    case 8: memcpy(out, s->sortedCellId.data(), n * sizeof(int)); break;
    case 9: memcpy(out, s->rotations.data(), s->rotations.size() * sizeof(float4)); break;
    case 10: memcpy(out, s->cms.data(), s->cms.size() * sizeof(float3)); break;
    case 11: memcpy(out, s->omegas.data(), n * sizeof(float3)); break;
    case 12: memcpy(out, s->normals.data(), n * sizeof(float3)); break;
    case 13: memcpy(out, s->m.data(), n * sizeof(float)); break;
    case 14: memcpy(out, s->phase.data(), n * sizeof(int)); break;
    default: return 1;
    }
    return 0;
}

/* Stand-alone grid: updateGridId + stable sort + findStartEndId on host arrays.
 * cell_start/cell_end: D^3 entries, -1 on entry. */
int ref_grid_build(int n, const float *pos, float cell, int D, int *cell_ids, int *sorted_cell_ids,
                   int *sorted_particle_ids, int *cell_start, int *cell_end)
{
    GridDim = (uint)D;
    GridCellSize = make_float3(cell);
    std::vector<float3> p(n);
    for (int i = 0; i < n; ++i) p[i] = make_float3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    std::vector<int> pid(n);
    const float3 *pp = p.data();
    int *pi = pid.data();
    float3 cellOrigin = make_float3(0.f);
    int3 gridSize = make_int3(D);
    float3 cs = make_float3(cell);
    launch(n, [&] { updateGridId(cell_ids, pi, pp, cellOrigin, cs, gridSize, n); });
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cell_ids[a] < cell_ids[b]; });
    for (int i = 0; i < n; ++i) {
        sorted_cell_ids[i] = cell_ids[order[i]];
        sorted_particle_ids[i] = pid[order[i]];
    }
    launch(n, [&] { findStartEndId(cell_start, cell_end, sorted_cell_ids, n); });
    return 0;
}

/* Neighbour counts with the reference's 27-cell loop (fluid.cuh:104-141
 * structure, counting instead of summing): sorted positions p, start/end tables. */
int ref_neighbor_counts(int n, const float *pos, float cell, int D, float h, const int *cell_start,
                        const int *cell_end, int *counts)
{
    GridDim = (uint)D;
    GridCellSize = make_float3(cell);
    SetKernelRadius(h);
    std::vector<float3> p(n);
    for (int i = 0; i < n; ++i) p[i] = make_float3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    launch(n, [&] {
        const int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
        if (i >= n) return;
        const int3 c = calcGridPos(p[i]);
        int cnt = 0;
        for (int z = c.z - 1; z <= c.z + 1; z++)
            for (int y = c.y - 1; y <= c.y + 1; y++)
                for (int x = c.x - 1; x <= c.x + 1; x++) {
                    const int a = calcGridAddress(x, y, z);
                    for (int j = cell_start[a]; j < cell_end[a]; j++)
                        if (length2(p[i] - p[j]) <= KernelSquaredRadius) cnt++;
                }
        counts[i] = cnt;
    });
    return 0;
}

}  /* extern "C" */
