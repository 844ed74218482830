/*
 * ref_cuda.cu -- brass-pan's OWN step on the GPU: the reference's kernel
 * headers compiled unmodified by nvcc for sm_103a and launched in the order of
 * ParticleSolver::update() (particlesolver.cuh:772-1072).
 *
 * TEST AND MEASUREMENT INFRASTRUCTURE (the reference's CUDA build,
 * "oracle/_ref/libbrassref_cuda.so"): it is the comparator the GB300 solver
 * is timed against and checked with, never part of the product.  The kernels
 * (brasstower/kernel/{util,grid,fluid,particleplane,particleparticle,distance,
 * wind,shapematching,immovable,bending}.cuh, with cuda/cudamatrix.cuh and
 * ext/helper_math.h) are read from the reference checkout or its staged copy
 * (see oracle/Makefile); oracle/refshim_cuda/ only blanks the OpenGL, console
 * and scene headers they include and nothing else.  CUB is the toolkit's.
 *
 * What is ours here is the replay, the same one oracle/ref_driver.cpp runs on
 * the host:
 *   - launches as the reference writes them: 128-thread blocks from
 *     GetNumBlocksNumThreads (kernel/util.cuh:3-8), one block of
 *     NUM_MAX_PARTICLE_PER_RIGID_BODY threads per rigid body, all on the
 *     legacy default stream;
 *   - updateGrid (particlesolver.cuh:712-765) with cub::DeviceRadixSort::SortPairs;
 *   - the commented constraint block (:881-993) and wind block (:838-858)
 *     enabled per stage bit, the solver-iteration count (hard-coded 2 at
 *     :862) as a parameter, and MASS_SCALING_CONSTANT (:809) as a parameter;
 *   - the one-line kernels defined inside particlesolver.cuh (which also holds
 *     host code nvcc cannot take: conio.h, MSVC-only exception constructors),
 *     restated below with their line numbers;
 *   - lambdas zeroed before every fluidLambda launch, so a solid's lambda,
 *     which fluidPosition reads (fluid.cuh:207) and fluidLambda never writes,
 *     is 0 as in the C restatement instead of left over from earlier passes.
 */
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <vector>

cudaError_t g_ref_cuda_first_error = cudaSuccess;

#include "kernel/util.cuh"
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

/* ---- one-line kernels of particlesolver.cuh, restated ------------------- */

__global__ void rc_applyGravity(float3 *p, int n, float dt) /* particlesolver.cuh:49-57 */
{
    int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
    if (i >= n) return;
    p[i] += make_float3(0.0f, -9.8f, 0.0f) * dt * dt;
}

__global__ void rc_predictPositions(float3 *np, const float3 *x, const float3 *v, int n, float dt) /* :59-69 */
{
    int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
    if (i >= n) return;
    np[i] = x[i] + v[i] * dt;
}

__global__ void rc_updateVelocity(float3 *v, const float3 *np, const float3 *x, int n, float invDt) /* :71-81 */
{
    int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
    if (i >= n) return;
    v[i] = (np[i] - x[i]) * invDt;
}

__global__ void rc_computeInvScaledMasses(float *w, const float *m, const float3 *x, float k, int n) /* :84-98 */
{
    int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
    if (i >= n) return;
    const float e = 2.7182818284f;
    const float height = x[i].y;
    const float scale = pow(e, -k * height);
    w[i] = 1.0f / (scale * m[i]);
}

__global__ void rc_updatePositions(float3 *x, const float3 *np, const int *phases, float thr, int n) /* :121-137 */
{
    int i = threadIdx.x + __mul24(blockIdx.x, blockDim.x);
    if (i >= n) return;
    const float3 xi = x[i];
    const float3 nx = np[i];
    const float d2 = length2(nx - xi);
    x[i] = (d2 >= thr * thr || phases[i] < 0) ? nx : xi;
}

/* Puts a state given in original order back into the identity arrangement. */
__global__ void rc_load_original(float3 *x, float3 *v, float *m, int *phase, int *group, int *toOrig, int *toNew,
                                 const float3 *hx, const float3 *hv, const float *m0, const int *ph0, const int *g0,
                                 int n)
{
    int i = threadIdx.x + blockIdx.x * blockDim.x;
    if (i >= n) return;
    x[i] = hx[i];
    v[i] = hv[i];
    m[i] = m0[i];
    phase[i] = ph0[i];
    group[i] = g0[i];
    toOrig[i] = i;
    toNew[i] = i;
}

/* ---- the solver state, mirroring ParticleSolver's device arrays --------- */

template <class T>
static T *dalloc(size_t count)
{
    T *p = nullptr;
    if (count == 0) count = 1;
    if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, count * sizeof(T));
    return p;
}

template <class T>
static T *dupload(const std::vector<T> &h, size_t extra = 0)
{
    T *p = dalloc<T>(h.size() + extra);
    if (p && !h.empty()) cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return p;
}

struct RefCuda {
    int n = 0, D = 0;
    float radius = 0, h = 0, cell = 0, restDensity = 0, massScalingK = 2.0f;
    /* device state (sorted order; std::swap'ed exactly like the reference) */
    float3 *x = nullptr, *p = nullptr, *v = nullptr, *sx = nullptr, *sp = nullptr, *sv = nullptr;
    float3 *dX = nullptr, *tmp = nullptr, *omegas = nullptr, *normals = nullptr;
    float *m = nullptr, *sm = nullptr, *w = nullptr, *lambdas = nullptr, *densities = nullptr;
    int *phase = nullptr, *sphase = nullptr, *group = nullptr, *sgroup = nullptr;
    int *toOrig = nullptr, *stoOrig = nullptr, *toNew = nullptr;
    int *cellId = nullptr, *particleId = nullptr, *sortedCellId = nullptr, *sortedParticleId = nullptr;
    int *cellStart = nullptr, *cellEnd = nullptr;
    void *temp = nullptr;
    size_t tempBytes = 0;
    /* constraints (original ids) */
    int nPairs = 0, nFaces = 0, nBodies = 0, nImm = 0, nBends = 0;
    int2 *pairs = nullptr, *ranges = nullptr;
    float2 *dparams = nullptr;
    int3 *faces = nullptr;
    int *imm = nullptr;
    int4 *bends = nullptr;
    float3 *rest = nullptr, *cms = nullptr;
    float4 *rot = nullptr;
    std::vector<float3> planeO, planeN;
    /* the scene's per-particle constants in original order (for set_state) */
    float *m0 = nullptr;
    int *ph0 = nullptr, *g0 = nullptr;
    float3 *hx = nullptr, *hv = nullptr;
};

static void blocks_for(int count, int *nb, int *nt) { GetNumBlocksNumThreads(nb, nt, count); }

static void set_constants(const RefCuda &s)
{
    SetKernelRadius(s.h); /* fluid.cuh:11-27, the reference's own host code */
    const uint D = (uint)s.D;
    const float3 cs = make_float3(s.cell);
    checkCudaErrors(cudaMemcpyToSymbol(GridDim, &D, sizeof(D)));
    checkCudaErrors(cudaMemcpyToSymbol(GridCellSize, &cs, sizeof(cs)));
}

/* updateGrid (particlesolver.cuh:712-765) */
static void update_grid(RefCuda &s, int nb, int nt)
{
    const int n = s.n;
    const float3 cellOrigin = make_float3(0.f);
    const float3 cellSize = make_float3(s.cell);
    const int3 gridSize = make_int3(s.D);
    updateGridId<<<nb, nt>>>(s.cellId, s.particleId, s.p, cellOrigin, cellSize, gridSize, n);
    size_t bytes = s.tempBytes;
    cub::DeviceRadixSort::SortPairs(s.temp, bytes, s.cellId, s.sortedCellId, s.particleId, s.sortedParticleId, n);
    findStartEndId<<<nb, nt>>>(s.cellStart, s.cellEnd, s.sortedCellId, n);
    reorderParticlesData<<<nb, nt>>>(s.sp, s.sx, s.sv, s.sm, s.sphase, s.stoOrig, s.sgroup, s.p, s.x, s.v, s.m,
                                     s.phase, s.group, s.toOrig, s.sortedParticleId, n);
    std::swap(s.sp, s.p);
    std::swap(s.sx, s.x);
    std::swap(s.sv, s.v);
    std::swap(s.sm, s.m);
    std::swap(s.sphase, s.phase);
    std::swap(s.sgroup, s.group);
    std::swap(s.stoOrig, s.toOrig);
}

/* setParticle (particlesolver.cuh:388-393) with the index looked up on the host */
static int new_id(RefCuda &s, int original)
{
    int id = -1;
    cudaMemcpy(&id, s.toNew + original, sizeof(int), cudaMemcpyDeviceToHost);
    return id;
}

static void set_particle(RefCuda &s, float3 *pos, int idx, float3 pp, float3 vel)
{
    if (idx < 0 || idx >= s.n) return;
    setDevArr_float3<<<1, 1>>>(pos + idx, pp, 1);
    setDevArr_float3<<<1, 1>>>(s.v + idx, vel, 1);
}

static void update(RefCuda &s, int numSub, float dt, int iterations, int mask, int picked, float3 pickedPos,
                   float3 pickedVel)
{
    if (s.n <= 0) return;
    const int n = s.n;
    int nb, nt;
    blocks_for(n, &nb, &nt);
    const float subDt = dt / (float)numSub;
    const bool useAkinci = (mask & BP_STAGE_AKINCI) != 0; /* hard-coded true (:785) */
    const float r = s.radius;
    for (int sub = 0; sub < numSub; ++sub) {
        if (picked >= 0 && picked < n) set_particle(s, s.x, new_id(s, picked), pickedPos, make_float3(0.f));

        rc_predictPositions<<<nb, nt>>>(s.p, s.x, s.v, n, subDt);
        rc_applyGravity<<<nb, nt>>>(s.p, n, subDt);
        update_grid(s, nb, nt);
        inverseMapping<<<nb, nt>>>(s.toNew, s.toOrig, n);
        rc_computeInvScaledMasses<<<nb, nt>>>(s.w, s.m, s.x, s.massScalingK, n);

        if (mask & BP_STAGE_PLANES)
            for (int it = 0; it < 2; ++it) /* :822-833 */
                for (size_t k = 0; k < s.planeO.size(); ++k)
                    planeStabilize<<<nb, nt>>>(s.x, s.p, n, s.planeO[k], s.planeN[k], r);

        if ((mask & BP_STAGE_WIND) && s.nFaces > 0) { /* :838-858 */
            int fb, ft;
            blocks_for(s.nFaces, &fb, &ft);
            setDevArr_float3<<<nb, nt>>>(s.dX, make_float3(0.f), n);
            applyWindForce<<<fb, ft>>>(s.dX, s.p, s.v, s.m, s.toNew, s.faces, s.nFaces, subDt);
            accDevArr_float3<<<nb, nt>>>(s.p, s.dX, n);
        }

        for (int j = 0; j < iterations; ++j) { /* :862-994 */
            if (picked >= 0 && picked < n) set_particle(s, s.p, new_id(s, picked), pickedPos, make_float3(0.f));
            if (mask & BP_STAGE_PLANES)
                for (size_t k = 0; k < s.planeO.size(); ++k)
                    particlePlaneCollisionConstraint<<<nb, nt>>>(s.p, s.x, n, s.planeO[k], s.planeN[k], r);
            if (mask & BP_STAGE_PARTICLE_COLLISION) {
                setDevArr_float3<<<nb, nt>>>(s.dX, make_float3(0.f), n);
                particleParticleCollisionConstraint<<<nb, nt>>>(s.dX, s.p, s.x, s.w, s.phase, s.cellStart,
                                                                s.cellEnd, n, r);
                accDevArr_float3<<<nb, nt>>>(s.p, s.dX, n);
            }
            if (mask & BP_STAGE_FLUID) {
                setDevArr_float<<<nb, nt>>>(s.lambdas, 0.0f, n);
                fluidLambda<<<nb, nt>>>(s.lambdas, s.densities, s.p, s.m, s.phase, s.restDensity, 2.0f, 300.0f,
                                        s.cellStart, s.cellEnd, n, useAkinci);
                setDevArr_float3<<<nb, nt>>>(s.dX, make_float3(0.f), n);
                fluidPosition<<<nb, nt>>>(s.dX, s.p, s.lambdas, s.restDensity, s.m, s.phase, 0.0001f, 4,
                                          s.cellStart, s.cellEnd, n, useAkinci);
                accDevArr_float3<<<nb, nt>>>(s.p, s.dX, n);
            }
            if ((mask & BP_STAGE_DISTANCE) && s.nPairs > 0) {
                int db, dt_;
                blocks_for(s.nPairs, &db, &dt_);
                setDevArr_float3<<<nb, nt>>>(s.dX, make_float3(0.f), n);
                distanceConstraints<<<db, dt_>>>(s.dX, s.p, s.w, s.pairs, s.dparams, s.toNew, s.nPairs);
                accDevArr_float3<<<nb, nt>>>(s.p, s.dX, n);
            }
            if ((mask & BP_STAGE_BENDING) && s.nBends > 0) { /* :956-969 */
                int bb, bt;
                blocks_for(s.nBends, &bb, &bt);
                setDevArr_float3<<<nb, nt>>>(s.dX, make_float3(0.f), n);
                bendingConstraints<<<bb, bt>>>(s.dX, s.p, s.w, s.bends, s.toNew, s.nBends);
                accDevArr_float3<<<nb, nt>>>(s.p, s.dX, n);
            }
            if ((mask & BP_STAGE_SHAPE_MATCHING) && s.nBodies > 0)
                shapeMatchingAlphaOne<<<s.nBodies, NUM_MAX_PARTICLE_PER_RIGID_BODY>>>(
                    s.rot, s.cms, s.p, s.toNew, s.rest, s.ranges);
            if ((mask & BP_STAGE_IMMOVABLE) && s.nImm > 0) {
                int ib, it_;
                blocks_for(s.nImm, &ib, &it_);
                immovableConstraints<<<ib, it_>>>(s.p, s.x, s.imm, s.toNew, s.nImm);
            }
        }

        rc_updateVelocity<<<nb, nt>>>(s.v, s.p, s.x, n, 1.0f / subDt);
        rc_updatePositions<<<nb, nt>>>(s.x, s.p, s.phase, PARTICLE_SLEEPING_EPSILON, n);

        if (mask & BP_STAGE_VORTICITY) {
            fluidOmega<<<nb, nt>>>(s.omegas, s.v, s.p, s.phase, s.cellStart, s.cellEnd, n);
            fluidVorticity<<<nb, nt>>>(s.v, s.omegas, s.p, 0.001f, s.phase, s.cellStart, s.cellEnd, n, subDt);
        }
        if (useAkinci) {
            fluidNormal<<<nb, nt>>>(s.normals, s.p, s.densities, s.phase, s.cellStart, s.cellEnd, n);
            fluidAkinciTension<<<nb, nt>>>(s.tmp, s.v, s.p, s.normals, s.densities, s.restDensity, s.phase, 0.5f,
                                           s.cellStart, s.cellEnd, n, subDt);
            std::swap(s.v, s.tmp);
        }
        if (mask & BP_STAGE_XSPH) {
            fluidXSph<<<nb, nt>>>(s.tmp, s.v, s.p, 0.0002f, s.phase, s.cellStart, s.cellEnd, n);
            std::swap(s.v, s.tmp);
        }
        resetStartEndId<<<nb, nt>>>(s.cellStart, s.cellEnd, s.sortedCellId, n);
    }
    if (picked >= 0 && picked < n) {
        const int id = new_id(s, picked);
        float3 xp;
        cudaMemcpy(&xp, s.x + id, sizeof(float3), cudaMemcpyDeviceToHost);
        set_particle(s, s.x, id, xp, pickedVel);
    }
}

static void release(RefCuda *s)
{
    void *ptrs[] = {s->x, s->p, s->v, s->sx, s->sp, s->sv, s->dX, s->tmp, s->omegas, s->normals, s->m, s->sm,
                    s->w, s->lambdas, s->densities, s->phase, s->sphase, s->group, s->sgroup, s->toOrig,
                    s->stoOrig, s->toNew, s->cellId, s->particleId, s->sortedCellId, s->sortedParticleId,
                    s->cellStart, s->cellEnd, s->temp, s->pairs, s->ranges, s->dparams, s->faces, s->imm,
                    s->bends, s->rest, s->cms, s->rot, s->m0, s->ph0, s->g0, s->hx, s->hv};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete s;
}

/* ---- C ABI for the Python tests and bench ------------------------------- */

extern "C" {

/* First CUDA error seen by the driver (0 when none); clears it. */
int refcu_error(void)
{
    cudaError_t e = g_ref_cuda_first_error;
    if (e == cudaSuccess) e = cudaGetLastError();
    g_ref_cuda_first_error = cudaSuccess;
    return (int)e;
}

void *refcu_create(const bp_scene_desc *sc, float radius, float h, float cell, int D, float restDensity,
                   float massScalingK)
{
    RefCuda *s = new RefCuda();
    const int n = sc->num_particles;
    s->n = n;
    s->D = D;
    s->radius = radius;
    s->h = h;
    s->cell = cell;
    s->restDensity = restDensity;
    s->massScalingK = massScalingK;
    auto f3 = [](const float *a, int i) { return make_float3(a[3 * i], a[3 * i + 1], a[3 * i + 2]); };
    std::vector<float3> x(n), v(n);
    std::vector<float> m(n);
    std::vector<int> ph(n), g(n, 0), iota(n);
    for (int i = 0; i < n; ++i) {
        x[i] = f3(sc->positions, i);
        v[i] = sc->velocities ? f3(sc->velocities, i) : make_float3(0.f);
        m[i] = sc->masses[i];
        ph[i] = sc->phases[i];
        if (sc->group_ids) g[i] = sc->group_ids[i];
        iota[i] = i;
    }
    s->x = dupload(x);
    s->p = dupload(x);
    s->v = dupload(v);
    s->sx = dalloc<float3>(n);
    s->sp = dalloc<float3>(n);
    s->sv = dalloc<float3>(n);
    s->dX = dalloc<float3>(n);
    s->tmp = dalloc<float3>(n);
    s->omegas = dalloc<float3>(n);
    s->normals = dalloc<float3>(n);
    s->m = dupload(m);
    s->sm = dalloc<float>(n);
    s->w = dalloc<float>(n);
    s->lambdas = dalloc<float>(n);
    s->densities = dalloc<float>(n);
    s->phase = dupload(ph);
    s->sphase = dalloc<int>(n);
    s->group = dupload(g);
    s->sgroup = dalloc<int>(n);
    s->toOrig = dupload(iota);
    s->stoOrig = dalloc<int>(n);
    s->toNew = dupload(iota, NUM_MAX_PARTICLE_PER_RIGID_BODY); /* shapeMatchingAlphaOne reads past a body's end */
    s->cellId = dalloc<int>(n);
    s->particleId = dalloc<int>(n);
    s->sortedCellId = dalloc<int>(n);
    s->sortedParticleId = dalloc<int>(n);
    const size_t cells = (size_t)D * D * D;
    s->cellStart = dalloc<int>(cells);
    s->cellEnd = dalloc<int>(cells);
    cudaMemset(s->cellStart, 0xff, cells * sizeof(int)); /* -1: the tables start empty */
    cudaMemset(s->cellEnd, 0xff, cells * sizeof(int));
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, s->cellId, s->sortedCellId, s->particleId, s->sortedParticleId,
                                    n);
    s->temp = dalloc<char>(bytes);
    s->tempBytes = bytes;
    for (int k = 0; k < sc->num_planes; ++k) {
        s->planeO.push_back(f3(sc->planes + 6 * k, 0));
        s->planeN.push_back(f3(sc->planes + 6 * k + 3, 0));
    }
    std::vector<int2> pairs;
    std::vector<float2> dparams;
    for (int k = 0; k < sc->num_distance_constraints; ++k) {
        pairs.push_back(make_int2(sc->distance_pairs[2 * k], sc->distance_pairs[2 * k + 1]));
        dparams.push_back(make_float2(sc->distance_params[2 * k], sc->distance_params[2 * k + 1]));
    }
    s->nPairs = (int)pairs.size();
    s->pairs = dupload(pairs);
    s->dparams = dupload(dparams);
    std::vector<int3> faces;
    for (int k = 0; k < sc->num_wind_faces; ++k)
        faces.push_back(make_int3(sc->wind_faces[3 * k], sc->wind_faces[3 * k + 1], sc->wind_faces[3 * k + 2]));
    s->nFaces = (int)faces.size();
    s->faces = dupload(faces);
    std::vector<int2> ranges;
    for (int k = 0; k < sc->num_rigid_bodies; ++k)
        ranges.push_back(make_int2(sc->rigid_ranges[2 * k], sc->rigid_ranges[2 * k + 1]));
    s->nBodies = (int)ranges.size();
    s->ranges = dupload(ranges);
    std::vector<float3> rest(n, make_float3(0.f));
    if (sc->rigid_rest_positions)
        for (int i = 0; i < n; ++i) rest[i] = f3(sc->rigid_rest_positions, i);
    s->rest = dupload(rest, NUM_MAX_PARTICLE_PER_RIGID_BODY);
    std::vector<float4> rot(ranges.size(), make_float4(0.f, 0.f, 0.f, 1.f));
    s->rot = dupload(rot);
    s->cms = dalloc<float3>(ranges.size());
    std::vector<int> imm(sc->immovables, sc->immovables + sc->num_immovables);
    s->nImm = (int)imm.size();
    s->imm = dupload(imm);
    std::vector<int4> bends;
    for (int k = 0; k < sc->num_bendings; ++k)
        bends.push_back(make_int4(sc->bendings[4 * k], sc->bendings[4 * k + 1], sc->bendings[4 * k + 2],
                                  sc->bendings[4 * k + 3]));
    s->nBends = (int)bends.size();
    s->bends = dupload(bends);
    s->m0 = dupload(m);
    s->ph0 = dupload(ph);
    s->g0 = dupload(g);
    s->hx = dalloc<float3>(n);
    s->hv = dalloc<float3>(n);
    if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess || !s->x || !s->temp ||
        !s->cellStart) {
        release(s);
        return nullptr;
    }
    return s;
}

void refcu_destroy(void *h)
{
    if (h) {
        cudaDeviceSynchronize();
        release((RefCuda *)h);
    }
}

/* Enqueues update() on the legacy default stream (no synchronisation unless
 * picking, which the reference also does through synchronous copies). */
int refcu_update(void *h, int numSub, float dt, int iterations, int mask, int picked, const float *pp,
                 const float *pv)
{
    RefCuda *s = (RefCuda *)h;
    set_constants(*s);
    float3 p = pp ? make_float3(pp[0], pp[1], pp[2]) : make_float3(0.f);
    float3 v = pv ? make_float3(pv[0], pv[1], pv[2]) : make_float3(0.f);
    update(*s, numSub, dt, iterations, mask, picked, p, v);
    return refcu_error();
}

/* `frames` updates, each preceded by a write of `flush_bytes` to `flush` (to
 * evict the state from L2) outside the timed interval; CUDA events on the
 * legacy default stream around each update.  Returns the summed milliseconds
 * in *ms_out. */
int refcu_time_updates(void *h, int frames, int numSub, float dt, int iterations, int mask, void *flush,
                       size_t flush_bytes, float *ms_out)
{
    RefCuda *s = (RefCuda *)h;
    set_constants(*s);
    std::vector<cudaEvent_t> ev(2 * (size_t)frames);
    for (auto &e : ev) cudaEventCreate(&e);
    cudaDeviceSynchronize();
    for (int f = 0; f < frames; ++f) {
        if (flush && flush_bytes) cudaMemsetAsync(flush, f & 0xff, flush_bytes, 0);
        cudaEventRecord(ev[2 * f], 0);
        update(*s, numSub, dt, iterations, mask, -1, make_float3(0.f), make_float3(0.f));
        cudaEventRecord(ev[2 * f + 1], 0);
    }
    cudaDeviceSynchronize();
    float total = 0.f;
    for (int f = 0; f < frames; ++f) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[2 * f], ev[2 * f + 1]);
        total += ms;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    *ms_out = total;
    return refcu_error();
}

/* Overwrites positions and velocities with host arrays in original order and
 * puts the particles back in original order (the tables stay as the last
 * substep's resetStartEndId left them: empty). */
int refcu_set_state(void *h, const float *x_orig, const float *v_orig)
{
    RefCuda *s = (RefCuda *)h;
    const size_t bytes = (size_t)s->n * sizeof(float3);
    cudaDeviceSynchronize();
    cudaMemcpy(s->hx, x_orig, bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(s->hv, v_orig, bytes, cudaMemcpyHostToDevice);
    rc_load_original<<<(s->n + 255) / 256, 256>>>(s->x, s->v, s->m, s->phase, s->group, s->toOrig, s->toNew, s->hx,
                                                  s->hv, s->m0, s->ph0, s->g0, s->n);
    cudaMemcpy(s->p, s->x, bytes, cudaMemcpyDeviceToDevice);
    cudaDeviceSynchronize();
    return refcu_error();
}

/* field ids as ref_get (ref_driver.cpp): 0 x, 1 p, 2 v (float3 [N]); 3 toOrig,
 * 4 toNew (int [N]); 5 lambdas, 6 densities, 7 invScaled (float [N]);
 * 8 sortedCellId (int [N]); 9 rotations (float4 [B]); 10 cms (float3 [B]);
 * 11 omegas, 12 normals (float3 [N]); 13 mass (float [N]); 14 phase (int [N]) */
int refcu_get(void *h, int field, void *out)
{
    RefCuda *s = (RefCuda *)h;
    const size_t n = (size_t)s->n, nb = (size_t)s->nBodies;
    cudaDeviceSynchronize();
    const void *src = nullptr;
    size_t bytes = 0;
    switch (field) {
    case 0: src = s->x; bytes = n * sizeof(float3); break;
    case 1: src = s->p; bytes = n * sizeof(float3); break;
    case 2: src = s->v; bytes = n * sizeof(float3); break;
    case 3: src = s->toOrig; bytes = n * sizeof(int); break;
    case 4: src = s->toNew; bytes = n * sizeof(int); break;
    case 5: src = s->lambdas; bytes = n * sizeof(float); break;
    case 6: src = s->densities; bytes = n * sizeof(float); break;
    case 7: src = s->w; bytes = n * sizeof(float); break;
    case 8: src = s->sortedCellId; bytes = n * sizeof(int); break;
    case 9: src = s->rot; bytes = nb * sizeof(float4); break;
    case 10: src = s->cms; bytes = nb * sizeof(float3); break;
    case 11: src = s->omegas; bytes = n * sizeof(float3); break;
    case 12: src = s->normals; bytes = n * sizeof(float3); break;
    case 13: src = s->m; bytes = n * sizeof(float); break;
    case 14: src = s->phase; bytes = n * sizeof(int); break;
    default: return -1;
    }
    if (bytes) cudaMemcpy(out, src, bytes, cudaMemcpyDeviceToHost);
    return refcu_error();
}

}  /* extern "C" */
