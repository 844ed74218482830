// bp_constraints.cu -- per-particle passes and the non-fluid constraints.
//
// Reference kernels (paths inside brass-pan, K/ = brasstower/kernel/):
//   particlePlaneCollisionConstraint (K/particleplane.cuh:21-58) -> k_planes
//   updateVelocity + updatePositions (particlesolver.cuh:71-81,121-137) -> k_commit
//   particleParticleCollisionConstraint (K/particleparticle.cuh:5-101) -> k_particle_collision
//   distanceConstraints (K/distance.cuh:3-40) -> k_distance_edges + k_distance_apply
//   bendingConstraints (K/bending.cuh:3-75)   -> k_bending_terms + k_bending_apply
//   applyWindForce (K/wind.cuh:3-50) -> k_wind_faces + k_wind_apply
//   shapeMatchingAlphaOne (K/shapematching.cuh:8-99) -> k_shape_matching (any body size)
//   immovableConstraints (K/immovable.cuh:3-14) -> k_immovable
//   mapParticleInfos (main.cu:273-282) -> k_pack_infos
// Scatter-with-atomics constraints become two deterministic passes: one
// thread per constraint computes its correction once, then one thread per
// affected particle sums its incident corrections in a fixed (CSR) order.
#include <algorithm>

#include "bp_internal.h"
#include "bp_walk.cuh"

namespace bp {

__global__ void k_planes(SimConsts C, const float4 *__restrict__ Xs, float4 *__restrict__ P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C.n) return;
    const float4 p4 = P[i];
    float3 p = f3(p4);
    plane_collide(C, scene_index(C, i), f3(Xs[i]), p);
    P[i] = make_float4(p.x, p.y, p.z, p4.w);
    track_displacement(C, i, p, true);
}

void launch_planes(cudaStream_t st, const SimConsts &C, const float4 *Xs, float4 *P, LaunchLog *L)
{
    if (C.n <= 0 || C.nplanes <= 0) return;
    k_planes<<<(C.n + 255) / 256, 256, 0, st>>>(C, Xs, P);
    L->done(__func__);
}

__global__ void k_commit(SimConsts C, const float4 *__restrict__ P, const float4 *__restrict__ Xs,
                         const float4 *__restrict__ Vs, const int *__restrict__ orig_s, float4 *__restrict__ Xc,
                         float4 *__restrict__ Vc, int *__restrict__ orig_c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C.n) return;
    const float4 p4 = P[i];
    const float4 xs = Xs[i];
    const float3 p = f3(p4);
    const float3 v = (p - f3(xs)) * C.inv_dt;
    Xc[i] = make_float4(p.x, p.y, p.z, xs.w);
    Vc[i] = make_float4(v.x, v.y, v.z, Vs[i].w);
    orig_c[i] = orig_s[i];
}

void launch_commit(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *Xs, const float4 *Vs,
                   const int *orig_s, float4 *Xc, float4 *Vc, int *orig_c, LaunchLog *L)
{
    if (C.n <= 0) return;
    k_commit<<<(C.n + 255) / 256, 256, 0, st>>>(C, P, Xs, Vs, orig_s, Xc, Vc, orig_c);
    L->done(__func__);
}

// ---- the solids of the cell-sorted order, compacted ----
// solid_prefix[i] = number of solids among sorted indices [0, i), for
// i in [0, n]; solid_list holds their sorted indices in order.  A column run
// [b, e) of the grid then holds the solids solid_list[prefix[b] .. prefix[e]).

constexpr int kScanBlock = 1024;

__global__ void __launch_bounds__(kScanBlock) k_solid_count(int n, const float4 *__restrict__ P, int *__restrict__ totals)
{
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const bool solid = i < n && phase_of(P[i]) > 0;
    const int c = __syncthreads_count(solid);
    if (threadIdx.x == 0) totals[blockIdx.x] = c;
}

// Exclusive scan of the block totals in one CTA (fixed order: deterministic).
__global__ void __launch_bounds__(kScanBlock) k_solid_scan_totals(int nb, int *__restrict__ totals,
                                                                   int *__restrict__ prefix, int n)
{
    __shared__ int part[kScanBlock];
    const int per = (nb + kScanBlock - 1) / kScanBlock;
    const int b0 = threadIdx.x * per, b1 = min(b0 + per, nb);
    int sum = 0;
    for (int b = b0; b < b1; ++b) sum += totals[b];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < kScanBlock; o <<= 1) {  // inclusive Hillis-Steele scan
        const int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int run = part[threadIdx.x] - sum;
    for (int b = b0; b < b1; ++b) {
        const int t = totals[b];
        totals[b] = run;
        run += t;
    }
    if (threadIdx.x == kScanBlock - 1) prefix[n] = part[kScanBlock - 1];
}

__global__ void __launch_bounds__(kScanBlock) k_solid_scatter(int n, const float4 *__restrict__ P,
                                                              const int *__restrict__ block_base,
                                                              int *__restrict__ prefix, int *__restrict__ list,
                                                              const int *__restrict__ keys,
                                                              unsigned long long *__restrict__ cells)
{
    __shared__ int warp_sum[kScanBlock / 32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const bool solid = i < n && phase_of(P[i]) > 0;
    const unsigned ballot = __ballot_sync(0xffffffffu, solid);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_sum[warp] = __popc(ballot);
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; ++w) before += warp_sum[w];
    const int pos = block_base[blockIdx.x] + before + __popc(ballot & ((1u << lane) - 1u));
    if (i < n) {
        prefix[i] = pos;
        if (solid) list[pos] = i;
    }
    if (solid && cells) {
        const unsigned key = (unsigned)__ldg(keys + i);
        atomicOr(cells + (key >> 6), 1ull << (key & 63u));
    }
}

// near[c] = some cell of the 27 around table cell c (the same masked
// neighbours a walk visits) stores a solid.  One thread per 64-bit word: with
// D >= 64 a word is 64 consecutive z of one (x, y) row, dilated in z by
// shifts and in x, y by the OR over the 9 rows; smaller grids test each bit.
__global__ void __launch_bounds__(256) k_solid_dilate(int D, int nwords, const unsigned long long *__restrict__ cells,
                                                      unsigned long long *__restrict__ near)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nwords) return;
    const unsigned m = (unsigned)D - 1u, DD = (unsigned)D * (unsigned)D;
    unsigned long long acc = 0ull;
    if (D >= 64) {
        const unsigned key0 = (unsigned)k * 64u, wpr = (unsigned)D / 64u;
        const unsigned x = key0 / DD, y = (key0 / (unsigned)D) & m, zw = (key0 & m) / 64u;
        const unsigned zp = (zw + wpr - 1u) % wpr, zn = (zw + 1u) % wpr;
        for (int r = 0; r < 9; ++r) {
            const unsigned rb = (((x + r / 3 - 1) & m) * DD + ((y + r % 3 - 1) & m) * (unsigned)D) / 64u;
            const unsigned long long w = __ldg(cells + rb + zw);
            acc |= w | (w << 1) | (w >> 1) | (__ldg(cells + rb + zp) >> 63) | (__ldg(cells + rb + zn) << 63);
        }
    } else {
        for (int b = 0; b < 64; ++b) {
            const unsigned key = (unsigned)k * 64u + (unsigned)b;
            const unsigned x = key / DD, y = (key / (unsigned)D) & m, z = key & m;
            bool any = false;
            for (int t = 0; t < 27 && !any; ++t) {
                const unsigned a = ((x + t / 9 - 1) & m) * DD + ((y + (t / 3) % 3 - 1) & m) * (unsigned)D +
                                   ((z + t % 3 - 1) & m);
                any = (__ldg(cells + (a >> 6)) >> (a & 63u)) & 1ull;
            }
            if (any) acc |= 1ull << b;
        }
    }
    near[k] = acc;
}

// The half of its cell p lies in on each axis (bit 0: x, 1: y, 2: z; set: the
// upper half, whose contact walks reach the next cell rather than the one
// before).
__device__ __forceinline__ int octant_of(float3 p, float cell)
{
    const float hc = 0.5f * cell;
    const int ox = cell_coord(__fsub_rn(p.x, hc), cell) == cell_coord(p.x, cell) ? 1 : 0;
    const int oy = cell_coord(__fsub_rn(p.y, hc), cell) == cell_coord(p.y, cell) ? 2 : 0;
    const int oz = cell_coord(__fsub_rn(p.z, hc), cell) == cell_coord(p.z, cell) ? 4 : 0;
    return ox | oy | oz;
}

// walk = the listed solids, each tile of 256 consecutive entries (cells in
// sorted order) regrouped by octant: the warps of a group take the same cells
// in their contact walks, and a tile's walks stay within its neighbourhood.
// The order within a group is any: every solid's result is its own.
__global__ void __launch_bounds__(256) k_solid_octant_tiles(int n, const int *__restrict__ prefix,
                                                            const int *__restrict__ list,
                                                            const float4 *__restrict__ P, float cell,
                                                            int *__restrict__ walk)
{
    __shared__ int h[8], base[8];
    const int total = __ldg(prefix + n);
    for (int t0 = blockIdx.x * blockDim.x; t0 < total; t0 += gridDim.x * blockDim.x) {  // uniform per CTA
        if (threadIdx.x < 8) h[threadIdx.x] = 0;
        __syncthreads();
        const int t = t0 + threadIdx.x;
        int o = -1, i = 0, rank = 0;
        if (t < total) {
            i = __ldg(list + t);
            o = octant_of(f3(P[i]), cell);
            rank = atomicAdd(&h[o], 1);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int run = 0;
            for (int q = 0; q < 8; ++q) {
                base[q] = run;
                run += h[q];
            }
        }
        __syncthreads();
        if (o >= 0) walk[t0 + base[o] + rank] = i;
        __syncthreads();
    }
}

void launch_solid_list(cudaStream_t st, int n, const float4 *P, int *totals, int *prefix, int *list,
                       const SolidCells &sc, LaunchLog *L, int nsolid, float cell, int *walk)
{
    if (n <= 0) return;
    const int nb = (n + kScanBlock - 1) / kScanBlock;
    const int nwords = sc.cells ? (int)((size_t)sc.D * sc.D * sc.D / 64) : 0;
    if (sc.cells) cudaMemsetAsync(sc.cells, 0, (size_t)nwords * sizeof(unsigned long long), st);
    k_solid_count<<<nb, kScanBlock, 0, st>>>(n, P, totals);
    L->done("k_solid_count");
    k_solid_scan_totals<<<1, kScanBlock, 0, st>>>(nb, totals, prefix, n);
    L->done("k_solid_scan_totals");
    k_solid_scatter<<<nb, kScanBlock, 0, st>>>(n, P, totals, prefix, list, sc.keys, sc.cells);
    L->done("k_solid_scatter");
    if (sc.cells) {
        k_solid_dilate<<<(nwords + 255) / 256, 256, 0, st>>>(sc.D, nwords, sc.cells, sc.near);
        L->done("k_solid_dilate");
    }
    if (walk && nsolid > 0) {  // sized by the count at creation, loops to the device total
        k_solid_octant_tiles<<<(nsolid + 255) / 256, 256, 0, st>>>(n, prefix, list, P, cell, walk);
        L->done("k_solid_octant_tiles");
    }
}

// ---- contact walks over the cells a partner can be stored in ----
// A contact partner j of walker i lies within 2r of p_i on every axis, and
// j's cell was hashed from a position at most d from p_j on every axis (d:
// C.contact_reach[0] over all particles, or [1] over the solids, the only
// partners of a fluid walker), so it is the cell of a point within 2r + d of
// p_i.  The cell
// function (float add and divide, truncation) is monotone, so on each axis
// that cell lies between the cells of p_i -+ (2r + d + margin); the margin
// covers the rounding of p_i -+ (...).  The range is clipped to the walker's
// 27 cells, which the full walk visits: both walks meet the same pairs in
// the same order.  A particle stored outside the range has no pair with i.

__device__ __forceinline__ bool contact_axis(float p, int c, float R, float cell, int &lo, int &hi)
{
    const float w = R + (1e-4f + fabsf(p) * 2.4e-7f);
    if (!(w < cell)) return false;  // also a NaN or infinite bound: the whole walk
    lo = max(cell_coord(__fsub_rn(p, w), cell) - c, -1);
    hi = min(cell_coord(__fadd_rn(p, w), cell) - c, 1);
    return true;
}

// The range of walker i at p (its cell c; fluid: it meets solids only); the
// whole 27 cells without a bound.
__device__ __forceinline__ CellRange contact_range(const SimConsts &C, float3 p, bool fluid)
{
    CellRange rg;
    if (!C.contact_reach) return rg;
    const float R = __fadd_rn(2.0f * C.radius, __uint_as_float(__ldg(C.contact_reach + (fluid ? 1 : 0))));
    const int3 c = cell_of(p, C);
    CellRange r;
    if (contact_axis(p.x, c.x, R, C.cell, r.lox, r.hix) && contact_axis(p.y, c.y, R, C.cell, r.loy, r.hiy) &&
        contact_axis(p.z, c.z, R, C.cell, r.loz, r.hiz))
        rg = r;
    return rg;
}

// The bounds: per axis, the largest |p - p_hash| over all particles (reach[0])
// and over the solids (reach[1]), positions P against the positions their
// cells were hashed from, as float bits (the maximum of non-negative floats is
// the maximum of their bits; a NaN's bits exceed every finite value's).
// reach[0..1] must be 0 before the launch.
__global__ void __launch_bounds__(256) k_contact_reach(int n, const float4 *__restrict__ P,
                                                       const float4 *__restrict__ hashed, unsigned *__restrict__ reach)
{
    unsigned best = 0u, best_solid = 0u;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = P[i], q = __ldg(hashed + i);
        const float d = fmaxf(fmaxf(fabsf(__fsub_rn(p.x, q.x)), fabsf(__fsub_rn(p.y, q.y))),
                              fabsf(__fsub_rn(p.z, q.z)));
        const bool finite = d <= 3.0e38f;
        const unsigned b = finite ? __float_as_uint(d) : 0x7f800000u;
        best = max(best, b);
        if (phase_of(p) > 0) best_solid = max(best_solid, b);
    }
    best = __reduce_max_sync(0xffffffffu, best);
    best_solid = __reduce_max_sync(0xffffffffu, best_solid);
    if ((threadIdx.x & 31) == 0 && best) atomicMax(reach, best);
    if ((threadIdx.x & 31) == 0 && best_solid) atomicMax(reach + 1, best_solid);
}

// The solids' bound only (reach[1]), over the compacted list; reach[0] = +inf
// (the solid walkers take all 27 cells).  reach[1] must be 0 before the launch.
__global__ void __launch_bounds__(256) k_contact_reach_solids(int n, const int *__restrict__ prefix,
                                                              const int *__restrict__ list,
                                                              const float4 *__restrict__ P,
                                                              const float4 *__restrict__ hashed,
                                                              unsigned *__restrict__ reach)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) reach[0] = 0x7f800000u;
    const int total = __ldg(prefix + n);
    unsigned best = 0u;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int i = __ldg(list + t);
        const float4 p = P[i], q = __ldg(hashed + i);
        const float d = fmaxf(fmaxf(fabsf(__fsub_rn(p.x, q.x)), fabsf(__fsub_rn(p.y, q.y))),
                              fabsf(__fsub_rn(p.z, q.z)));
        best = max(best, d <= 3.0e38f ? __float_as_uint(d) : 0x7f800000u);
    }
    best = __reduce_max_sync(0xffffffffu, best);
    if ((threadIdx.x & 31) == 0 && best) atomicMax(reach + 1, best);
}

void launch_contact_reach(cudaStream_t st, int n, const float4 *P, const float4 *hashed, unsigned *reach,
                          LaunchLog *L, int nsolid, const int *solid_prefix, const int *solid_list)
{
    cudaMemsetAsync(reach, 0, 2 * sizeof(unsigned), st);
    if (n <= 0) return;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (solid_list && 2LL * nsolid < n) {  // mostly fluid: bound the solids only
        const int blocks = std::min((std::max(nsolid, 1) + 255) / 256, std::max(sms, 1) * 8);
        k_contact_reach_solids<<<blocks, 256, 0, st>>>(n, solid_prefix, solid_list, P, hashed, reach);
        L->done("k_contact_reach_solids");
        return;
    }
    const int blocks = std::min((n + 255) / 256, std::max(sms, 1) * 8);
    k_contact_reach<<<blocks, 256, 0, st>>>(n, P, hashed, reach);
    L->done("k_contact_reach");
}

// The solids among the candidates of particle i's 27 cells (or of the cells
// of rg), in walk order: body(j, P[j]) for every solid j with test(-1, P[j])
// (a fluid walker: no candidate is itself).  spos[k] = P[list[k]]
// (k_gather_solids).
template <class T, class B>
__device__ __forceinline__ void walk_solids(float3 pi, const float4 *__restrict__ spos, const GridView &v,
                                            const SimConsts &C, const int *__restrict__ prefix,
                                            const int *__restrict__ list, T &&test, B &&body,
                                            CellRange rg = CellRange{})
{
    const int3 c = cell_of(pi, C);
    const unsigned m = v.mask, D = (unsigned)v.D;
    const unsigned z0 = (unsigned)(c.z + rg.loz) & m, z2 = (unsigned)(c.z + rg.hiz) & m;
    // a range of 3 cells never starts and ends on one table cell (D >= 4)
    const bool wrap = (rg.hiz - rg.loz == 2) ? !(z0 < z2) : z0 > z2;
#pragma unroll 1
    for (int col = 0; col < 9; ++col) {
        const int dx = col / 3 - 1, dy = col % 3 - 1;
        if (dx < rg.lox || dx > rg.hix || dy < rg.loy || dy > rg.hiy) continue;
        const unsigned x = (unsigned)(c.x + dx) & m, y = (unsigned)(c.y + dy) & m;
        const unsigned base = x * D * D + y * D;
#pragma unroll 1
        for (int piece = 0; piece < (wrap ? 2 : 1); ++piece) {
            const unsigned za = (wrap && piece == 1) ? 0u : z0;
            const unsigned zb = wrap ? (piece == 0 ? D - 1 : z2) : z2;
            const int b = __ldg(v.off + base + za), e = __ldg(v.off + base + zb + 1);
            const int kb = __ldg(prefix + b), ke = __ldg(prefix + e);
#pragma unroll 1
            for (int k = kb; k < ke; ++k) {
                // positions in list order (k_gather_solids); the sorted index
                // only for a hit (the walker is fluid, so no candidate is itself)
                const float4 pj = __ldg(spos + k);
                if (test(-1, pj)) body(__ldg(list + k), pj);
            }
        }
    }
}

// Solid contacts: pairs of different phase with at least one solid, closer
// than two radii; mass-weighted projection plus friction averaged over the
// counted contacts; only particle i moves (the reference's j update is
// commented out).  Reads P, writes Pout = P + delta.  A fluid particle only
// meets solids, so it walks the compacted solids of its 27 cells (same
// candidates in the same order; the others contribute nothing).
template <bool Split>
__device__ __forceinline__ void collide_one(const SimConsts &C, int i, const float4 *__restrict__ P,
                                            const float4 *__restrict__ Xs, const float *__restrict__ w,
                                            const GridView &v, const StageShared *S, int g,
                                            const int *__restrict__ solid_prefix, const int *__restrict__ solid_list,
                                            const float4 *__restrict__ solid_pos, float4 *__restrict__ Pout)
{
    const float4 pi4 = P[i];
    const float3 xip = f3(pi4);
    const int phi = phase_of(pi4);
    const float r = C.radius;
    const float3 xi = f3(Xs[i]);
    const float wi = w[i];
    float3 sd = make_float3(0.f, 0.f, 0.f), sf = make_float3(0.f, 0.f, 0.f);
    int count = 0;
    auto test = [&](int j, float4 pj4) {
        const int phj = phase_of(pj4);
        const float d2 = len2(xip - f3(pj4));
        return j != i && phi != phj && (phi > 0 || phj > 0) && d2 < r * r * 4.0f && d2 > 1e-5f;
    };
    auto body = [&](int j, float4 pj4) {
            const float3 xjp = f3(pj4);
            const float3 diff = xip - xjp;
            const float d2 = len2(diff);
            const float dist = __fsqrt_rn(d2);
            const float wj = w[j];
            const float w1 = __fdiv_rn(wi, __fadd_rn(wi, wj));
            const float w2 = __fdiv_rn(wj, __fadd_rn(wi, wj));
            const float3 proj = diff * __fsub_rn(__fdiv_rn(2.0f * r, dist), 1.0f);
            const float3 dxi = w1 * proj;
            const float3 xistar = dxi + xip;
            sd += dxi;
            const float3 dxj = -w2 * proj;
            const float dxi2 = len2(dxi);
            if (dxi2 > r * r * 0.001f * 0.001f) {
                count += 1;
                const float3 xj = f3(Xs[j]);
                const float3 xjstar = dxj + xjp;
                const float3 t1 = (xistar - xi) - (xjstar - xj);
                const float3 nn = diff / dist;
                const float3 tdx = t1 - dot3(t1, nn) * nn;
                const float tl2 = len2(tdx);
                if (tl2 <= __fmul_rn(C.fs * C.fs, dxi2))
                    sf -= w1 * tdx;
                else
                    sf -= (w1 * tdx) * fminf(__fmul_rn(C.fd, __fsqrt_rn(__fdiv_rn(dxi2, tl2))), 1.0f);
            }
    };
    const CellRange rg = contact_range(C, xip, phi < 0 && solid_prefix);
    if (phi < 0 && solid_prefix) walk_solids(xip, solid_pos, v, C, solid_prefix, solid_list, test, body, rg);
    else walk_neighbors<Split, true>(i, xip, 0, P, v, C, S, g, test, body, rg);
    const float3 d = (count == 0) ? sd : sd + sf / (float)count;
    const float3 p = xip + d;
    Pout[i] = make_float4(p.x, p.y, p.z, pi4.w);
    track_displacement(C, i, p, true);
}

// Fluid particles (and, without a solid list, everything), one CTA per 256
// sorted particles.  A CTA of fluid whose runs touch no tile holding a solid
// skips the walks: none of its particles that stayed in their stored cell
// can meet a solid.  So does a fluid particle whose current cell has no
// solid stored in its 27 cells (solid_near, k_solid_dilate): its walk over
// the solids would visit none.
template <bool Split>
__device__ __forceinline__ void k_particle_collision_tile(
    const SimConsts &C,
    const float4 *__restrict__ P,
    const float4 *__restrict__ Xs,
    const float *__restrict__ w,
    const int *__restrict__ off,
    const int *__restrict__ tile_solid,
    const int *__restrict__ solid_prefix,
    const int *__restrict__ solid_list,
    const float4 *__restrict__ solid_pos,
    const unsigned long long *__restrict__ solid_near,
    int solids_apart,
    float4 *__restrict__ Pout,
    int i0)
{
    StageShared &S = stage_shared();
    // With the solids apart, fluid threads walk the solid list, not the
    // staged runs: only the runs' solid check is needed.
    const int g = stage_block(C, P, off, i0, S, tile_solid, !solids_apart);
    const int i = i0 + threadIdx.x;
    if (i >= C.n) return;
    const float4 pi4 = P[i];
    const int phi = phase_of(pi4);
    if (phi > 0 && solids_apart) return;  // k_particle_collision_solids
    const GridView v = grid_view(C, scene_index(C, i), off);
    const float3 xip = f3(pi4);
    const int3 ci = cell_of(xip, C);
    const int cur_key = cell_addr(ci.x, ci.y, ci.z, v.D, v.mask);
    const bool in_cell = cur_key + v.base == __ldg(C.cell_keys + i);
    const bool none_near = solid_near && !((__ldg(solid_near + (cur_key >> 6)) >> (cur_key & 63)) & 1ull);
    if (phi < 0 && (none_near || (in_cell && (g == kNoSolidNear || (g >= 0 && !S.has_solid))))) {
        const float3 p = xip + make_float3(0.f, 0.f, 0.f);
        Pout[i] = make_float4(p.x, p.y, p.z, pi4.w);
        track_displacement(C, i, p, true);
        return;
    }
    collide_one<Split>(C, i, P, Xs, w, v, &S, g, solid_prefix, solid_list, solid_pos, Pout);
}

template <bool Split, bool Persist = false>
__global__ void __launch_bounds__(kWalkThreads, BP_SCAN_MIN_BLOCKS) k_particle_collision(
    SimConsts C,
    const float4 *__restrict__ P,
    const float4 *__restrict__ Xs,
    const float *__restrict__ w,
    const int *__restrict__ off,
    const int *__restrict__ tile_solid,
    const int *__restrict__ solid_prefix,
    const int *__restrict__ solid_list,
    const float4 *__restrict__ solid_pos,
    const unsigned long long *__restrict__ solid_near,
    int solids_apart,
    float4 *__restrict__ Pout)
{
    // one tile of blockDim.x particles per CTA, or, persistent (an unstaged
    // launch of at most one resident wave: SimConsts::scan_persist), every
    // gridDim.x-th tile from blockIdx.x on
    if constexpr (Persist) {
        for (int i0 = blockIdx.x * blockDim.x; i0 < C.n; i0 += gridDim.x * blockDim.x)
            k_particle_collision_tile<Split>(C, P, Xs, w, off, tile_solid, solid_prefix, solid_list, solid_pos,
                                             solid_near, solids_apart, Pout, i0);
    } else {
        k_particle_collision_tile<Split>(C, P, Xs, w, off, tile_solid, solid_prefix, solid_list, solid_pos,
                                         solid_near, solids_apart, Pout, blockIdx.x * blockDim.x);
    }
}

// The positions of the compacted solids, in list order, for the fluid
// walkers' reads (sequential within a run instead of a gather per candidate).
// The count is the device-side total of this substep's compaction
// (prefix[n]): phases can change after creation (a snapshot, a write through
// BP_FIELD_NEW_POSITIONS), so the launch's size, taken from the count at
// creation, is covered by a grid-stride loop.
__global__ void __launch_bounds__(256) k_gather_solids(int n, const int *__restrict__ prefix,
                                                       const int *__restrict__ list, const float4 *__restrict__ P,
                                                       float4 *__restrict__ spos)
{
    const int total = __ldg(prefix + n);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x)
        spos[k] = P[__ldg(list + k)];
}

// The solid particles, one thread each through the compacted list (in
// walk order: grouped by octant, so that a warp's contact walks take the same
// cells), so the long walks of solids scattered through fluid run in full
// warps.
template <bool Split>
__global__ void __launch_bounds__(kWalkThreads)
    k_particle_collision_solids(SimConsts C, int nsolid, const float4 *__restrict__ P,
                                const float4 *__restrict__ Xs, const float *__restrict__ w,
                                const int *__restrict__ off, const int *__restrict__ solid_prefix,
                                const int *__restrict__ solid_list, float4 *__restrict__ Pout)
{
    // the device-side count of this substep (see k_gather_solids); nsolid,
    // the count at creation, only sized the launch
    const int total = __ldg(solid_prefix + C.n);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int i = __ldg(solid_list + t);
        collide_one<Split>(C, i, P, Xs, w, grid_view(C, scene_index(C, i), off), nullptr, -1, nullptr, nullptr,
                           nullptr, Pout);
    }
}

void launch_particle_collision(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *Xs,
                               const float *w, const int *off, const int *tile_solid, const int *solid_prefix,
                               const int *solid_list, const int *solid_walk, int nsolid, bool solids_apart,
                               const unsigned long long *solid_near, float4 *solid_pos, float4 *Pout, LaunchLog *L)
{
    if (C.n <= 0) return;
    const int apart = (solids_apart && solid_prefix && solid_list && nsolid > 0) ? 1 : 0;
    // the cell mask describes the walks over the compacted solids only
    const unsigned long long *near = (apart && solid_prefix) ? solid_near : nullptr;
    if (solid_prefix && solid_list) {
        k_gather_solids<<<(max(nsolid, 1) + 255) / 256, 256, 0, st>>>(C.n, solid_prefix, solid_list, P, solid_pos);
        L->done("k_gather_solids");
    }
    if (C.split && !C.stage && C.scan_persist)
        launch_scan(k_particle_collision<true, true>, C, stage_bytes(C), st, C, P, Xs, w, off, tile_solid,
                    solid_prefix, solid_list, solid_pos, near, apart, Pout);
    else if (C.split)
        launch_scan(k_particle_collision<true>, C, stage_bytes(C), st, C, P, Xs, w, off, tile_solid, solid_prefix,
                    solid_list, solid_pos, near, apart, Pout);
    else
        launch_scan(k_particle_collision<false>, C, stage_bytes(C), st, C, P, Xs, w, off, tile_solid, solid_prefix,
                    solid_list, solid_pos, near, apart, Pout);
    L->done(__func__);
    if (apart) {  // the unstaged scans' CTA size (SimConsts::scan_block) here too
        const int sb = C.scan_block > 0 ? C.scan_block : kWalkThreads;
        const int sg = (nsolid + sb - 1) / sb;
        const int *order = solid_walk ? solid_walk : solid_list;
        if (C.split)
            k_particle_collision_solids<true><<<sg, sb, 0, st>>>(C, nsolid, P, Xs, w, off, solid_prefix, order, Pout);
        else
            k_particle_collision_solids<false><<<sg, sb, 0, st>>>(C, nsolid, P, Xs, w, off, solid_prefix, order, Pout);
        L->done("launch_particle_collision_solids");
    }
}

// ---- distance constraints ----

__global__ void k_distance_edges(int m, const int2 *__restrict__ pairs, const float2 *__restrict__ params,
                                 const float4 *__restrict__ P, const float *__restrict__ w,
                                 const int *__restrict__ to_new, float4 *__restrict__ edge_k)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    const int2 pr = pairs[e];
    const float2 prm = params[e];
    const int id1 = to_new[pr.x], id2 = to_new[pr.y];
    const float3 x12 = f3(P[id1]) - f3(P[id2]);
    const float d12 = len3(x12);
    float3 k = make_float3(0.f, 0.f, 0.f);
    if (!(d12 <= 1e-5f)) {
        const float3 nn = x12 / d12;
        const float sw = w[id1] + w[id2];
        k = (nn * ((d12 - prm.x) / sw)) * prm.y;
    }
    edge_k[e] = make_float4(k.x, k.y, k.z, 0.f);
}

__global__ void k_distance_apply(SimConsts C, int nn_, const int *__restrict__ node_ids, const int *__restrict__ ptr,
                                 const int *__restrict__ inc, const float4 *__restrict__ edge_k,
                                 const float *__restrict__ w, const int *__restrict__ to_new, float4 *__restrict__ P)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn_) return;
    const int i = to_new[node_ids[t]];
    const float wi = w[i];
    float3 d = make_float3(0.f, 0.f, 0.f);
    for (int q = ptr[t]; q < ptr[t + 1]; ++q) {
        const int code = inc[q];
        const float3 k = f3(edge_k[code >> 1]);
        d += (code & 1) ? wi * k : -wi * k;
    }
    const float4 p4 = P[i];
    const float3 p = make_float3(p4.x + d.x, p4.y + d.y, p4.z + d.z);
    P[i] = make_float4(p.x, p.y, p.z, p4.w);
    track_displacement(C, i, p, true);
}

void launch_distance(cudaStream_t st, const SimConsts &C, const DistanceArgs &a, float4 *P, const float *w,
                     const int *to_new, unsigned *err, LaunchLog *L)
{
    (void)err;
    if (a.num_edges <= 0) return;
    k_distance_edges<<<(a.num_edges + 255) / 256, 256, 0, st>>>(a.num_edges, a.pairs, a.params, P, w, to_new,
                                                                a.edge_k);
    L->done("k_distance_edges");
    k_distance_apply<<<(a.num_nodes + 255) / 256, 256, 0, st>>>(C, a.num_nodes, a.node_ids, a.node_ptr, a.node_inc,
                                                                a.edge_k, w, to_new, P);
    L->done("k_distance_apply");
}

// ---- dihedral bending ----

// bendingConstraints (K/bending.cuh:3-75): the dihedral angle of the two
// triangles (1, 2, 3) and (1, 2, 4) over the hinge 1-2 is pulled towards pi
// (flat) with the gradients of Mueller et al., Position Based Dynamics (2007),
// appendix A, in the reference's sequence of operations.  One thread per quad
// writes the four corrections; degenerate quads (a triangle normal or the
// denominator below 1e-5) write zeros, as the reference skips them.
__global__ void k_bending_terms(int nq, const int4 *__restrict__ quads, const float4 *__restrict__ P,
                                const float *__restrict__ w, const int *__restrict__ to_new, float kb,
                                float4 *__restrict__ terms)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int4 ids = quads[q];
    const int i1 = to_new[ids.x], i2 = to_new[ids.y], i3 = to_new[ids.z], i4 = to_new[ids.w];
    float4 *out = terms + 4 * (size_t)q;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    const float3 p1 = f3(P[i1]);
    const float3 e = f3(P[i2]) - p1, a = f3(P[i3]) - p1, b = f3(P[i4]) - p1;
    const float3 ca = cross3(e, a), cb = cross3(e, b);
    const float la = len3(ca), lb = len3(cb);
    if (la <= 1e-5f || lb <= 1e-5f) {
        out[0] = out[1] = out[2] = out[3] = zero;
        return;
    }
    const float3 n1 = ca * __fdiv_rn(1.0f, la), n2 = cb * __fdiv_rn(1.0f, lb);
    const float d = fminf(fmaxf(dot3(n1, n2), -1.0f), 1.0f);
    const float3 en1 = cross3(e, n1), en2 = cross3(e, n2);
    const float3 an1 = cross3(a, n1), an2 = cross3(a, n2);
    const float3 bn1 = cross3(b, n1), bn2 = cross3(b, n2);
    const float3 q3 = (en2 - en1 * d) / la;
    const float3 q4 = (en1 - en2 * d) / lb;
    const float3 q2 = -((an2 - an1 * d) / la) - (bn1 - bn2 * d) / lb;
    const float3 q1 = (-q2 - q3) - q4;
    const float w1 = w[i1], w2 = w[i2], w3 = w[i3], w4 = w[i4];
    const float den = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w1, len2(q1)), __fmul_rn(w2, len2(q2))),
                                          __fmul_rn(w3, len2(q3))),
                                __fmul_rn(w4, len2(q4)));
    const float num = __fmul_rn(__fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(d, d))), __fsub_rn(acosf(d), 3.141592f));
    if (den <= 1e-5f) {
        out[0] = out[1] = out[2] = out[3] = zero;
        return;
    }
    const float s = __fdiv_rn(num, den);
    const float3 d1 = ((-w1 * q1) * s) * kb, d2 = ((-w2 * q2) * s) * kb;
    const float3 d3 = ((-w3 * q3) * s) * kb, d4 = ((-w4 * q4) * s) * kb;
    out[0] = make_float4(d1.x, d1.y, d1.z, 0.f);
    out[1] = make_float4(d2.x, d2.y, d2.z, 0.f);
    out[2] = make_float4(d3.x, d3.y, d3.z, 0.f);
    out[3] = make_float4(d4.x, d4.y, d4.z, 0.f);
}

// Each particle with incident quads adds their corrections in CSR order (the
// reference's atomic scatter into deltaX, then accDevArr_float3).
__global__ void k_bending_apply(SimConsts C, int nn_, const int *__restrict__ node_ids, const int *__restrict__ ptr,
                                const int *__restrict__ inc, const float4 *__restrict__ terms,
                                const int *__restrict__ to_new, float4 *__restrict__ P)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn_) return;
    const int i = to_new[node_ids[t]];
    float3 d = make_float3(0.f, 0.f, 0.f);
    for (int q = ptr[t]; q < ptr[t + 1]; ++q) d += f3(terms[inc[q]]);
    const float4 p4 = P[i];
    const float3 p = f3(p4) + d;
    P[i] = make_float4(p.x, p.y, p.z, p4.w);
    track_displacement(C, i, p, true);
}

void launch_bending(cudaStream_t st, const SimConsts &C, const BendingArgs &a, float4 *P, const float *w,
                    const int *to_new, LaunchLog *L)
{
    if (a.num_quads <= 0) return;
    k_bending_terms<<<(a.num_quads + 255) / 256, 256, 0, st>>>(a.num_quads, a.quads, P, w, to_new, a.stiffness,
                                                              a.terms);
    L->done("k_bending_terms");
    k_bending_apply<<<(a.num_nodes + 255) / 256, 256, 0, st>>>(C, a.num_nodes, a.node_ids, a.node_ptr, a.node_inc,
                                                               a.terms, to_new, P);
    L->done("k_bending_apply");
}

// ---- wind ----

__global__ void k_wind_faces(SimConsts C, int nf, const int *__restrict__ faces, const float4 *__restrict__ P,
                             const float4 *__restrict__ V, const int *__restrict__ to_new,
                             float4 *__restrict__ move)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int id1 = to_new[faces[3 * f]], id2 = to_new[faces[3 * f + 1]], id3 = to_new[faces[3 * f + 2]];
    const float3 p1 = f3(P[id1]), p2 = f3(P[id2]), p3 = f3(P[id3]);
    const float3 a = p2 - p1, b = p3 - p1;
    float3 v = ((f3(V[id1]) + f3(V[id2])) + f3(V[id3])) / 3.f;
    if (C.textbook) v = v - C.wind;
    float3 mv = make_float3(0.f, 0.f, 0.f);
    const float lv = len3(v);
    if (!(lv <= 1e-5f)) {
        const float3 vh = v / lv;
        float3 fn = cross3(a, b);
        const float lf = len3(fn);
        if (!(lf <= 1e-5f)) {
            fn = fn / lf;
            fn = (dot3(fn, v) > 0.f) ? fn : -fn;
            const float area = 0.5f * lf;
            const float3 drag = (C.wind_drag * (lv * lv) * area * dot3(fn, vh)) * (-vh);
            const float3 uh = cross3(cross3(fn, vh), vh);
            const float3 lift = (C.wind_lift * (lv * lv) * area * dot3(fn, vh)) * uh;
            mv = ((drag + lift) * C.dt) * C.dt;
        }
    }
    move[f] = make_float4(mv.x, mv.y, mv.z, 0.f);
}

__global__ void k_wind_apply(SimConsts C, int nn_, const int *__restrict__ node_ids, const int *__restrict__ ptr,
                             const int *__restrict__ inc, const float4 *__restrict__ move,
                             const float *__restrict__ mass, const int *__restrict__ to_new, float4 *__restrict__ P)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn_) return;
    const int i = to_new[node_ids[t]];
    const float m = mass[i];
    float3 d = make_float3(0.f, 0.f, 0.f);
    for (int q = ptr[t]; q < ptr[t + 1]; ++q) d += f3(move[inc[q]]) / m;
    const float4 p4 = P[i];
    const float3 p = make_float3(p4.x + d.x, p4.y + d.y, p4.z + d.z);
    P[i] = make_float4(p.x, p.y, p.z, p4.w);
    track_displacement(C, i, p, true);
}

void launch_wind(cudaStream_t st, const SimConsts &C, const WindArgs &a, float4 *P, const float4 *Vs,
                 const float *mass, const int *to_new, LaunchLog *L)
{
    if (a.num_faces <= 0) return;
    k_wind_faces<<<(a.num_faces + 255) / 256, 256, 0, st>>>(C, a.num_faces, a.faces, P, Vs, to_new, a.face_move);
    L->done("k_wind_faces");
    k_wind_apply<<<(a.num_nodes + 255) / 256, 256, 0, st>>>(C, a.num_nodes, a.node_ids, a.node_ptr, a.node_inc,
                                                            a.face_move, mass, to_new, P);
    L->done("k_wind_apply");
}

// ---- shape matching ----

struct Quat { float x, y, z, w; };

__device__ __forceinline__ Quat qmul(Quat a, Quat b)
{
    Quat r;
    r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
    r.y = a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x;
    r.z = a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w;
    r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
    return r;
}

struct Mat3 { float3 c0, c1, c2; };

__device__ __forceinline__ Mat3 qmatrix(Quat q)
{
    const float x2 = q.x * q.x, y2 = q.y * q.y, z2 = q.z * q.z;
    Mat3 m;
    m.c0 = make_float3(1 - 2 * y2 - 2 * z2, 2 * q.x * q.y + 2 * q.w * q.z, 2 * q.x * q.z - 2 * q.w * q.y);
    m.c1 = make_float3(2 * q.x * q.y - 2 * q.w * q.z, 1 - 2 * x2 - 2 * z2, 2 * q.y * q.z + 2 * q.w * q.x);
    m.c2 = make_float3(2 * q.x * q.z + 2 * q.w * q.y, 2 * q.y * q.z - 2 * q.w * q.x, 1 - 2 * x2 - 2 * y2);
    return m;
}

constexpr int kSmThreads = 256;

// Block-wide sum of `nv` floats per thread (warp shuffles, then smem).
template <int NV>
__device__ __forceinline__ void block_sum(float (&v)[NV], float (*red)[32])
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        float s = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) red[k][warp] = s;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        float s = 0.f;
        for (int q = 0; q < kSmThreads / 32; ++q) s += red[k][q];
        v[k] = s;
    }
    __syncthreads();
}

// One CTA per body, any number of particles (looped in chunks of 256).
// Centre of mass (unweighted), A_pq columns, warm-started robust rotation
// extraction (Mueller et al. 2016, the reference's iteration with its
// 1/|sum| + 1e-9 denominator), goal positions with alpha = 1.
__global__ void __launch_bounds__(kSmThreads) k_shape_matching(SimConsts C, RigidArgs a, float4 *__restrict__ P,
                                                               const int *__restrict__ to_new)
{
    __shared__ float red[9][32];
    __shared__ float3 s_cm;
    __shared__ Mat3 s_R;
    const int b = blockIdx.x;
    const int2 rg = a.ranges[b];
    const int np = rg.y - rg.x;
    float c[3] = {0.f, 0.f, 0.f};
    for (int t = threadIdx.x; t < np; t += kSmThreads) {
        const float4 p = P[to_new[rg.x + t]];
        c[0] += p.x;
        c[1] += p.y;
        c[2] += p.z;
    }
    block_sum<3>(c, red);
    const float3 cm = make_float3(c[0], c[1], c[2]) / (float)np;
    float A[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int t = threadIdx.x; t < np; t += kSmThreads) {
        const float3 q = f3(a.rest[rg.x + t]);
        const float3 pc = f3(P[to_new[rg.x + t]]) - cm;
        A[0] += pc.x * q.x; A[1] += pc.y * q.x; A[2] += pc.z * q.x;
        A[3] += pc.x * q.y; A[4] += pc.y * q.y; A[5] += pc.z * q.y;
        A[6] += pc.x * q.z; A[7] += pc.y * q.z; A[8] += pc.z * q.z;
    }
    block_sum<9>(A, red);
    if (threadIdx.x == 0) {
        const float3 a0 = make_float3(A[0], A[1], A[2]), a1 = make_float3(A[3], A[4], A[5]),
                     a2 = make_float3(A[6], A[7], A[8]);
        const float4 q4 = a.rot[b];
        Quat q = {q4.x, q4.y, q4.z, q4.w};
        for (int it = 0; it < C.rot_iters; ++it) {
            const Mat3 R = qmatrix(q);
            const float3 num = (cross3(R.c0, a0) + cross3(R.c1, a1)) + cross3(R.c2, a2);
            const float den = 1.0f / fabsf(dot3(R.c0, a0) + dot3(R.c1, a1) + dot3(R.c2, a2)) + 1e-9f;
            const float3 om = num * den;
            const float w2 = len2(om);
            if (w2 <= 1e-9f) break;
            const float wl = sqrtf(w2);
            const float3 ax = om / wl;
            float sh, ch;
            sincosf(wl * 0.5f, &sh, &ch);
            const Quat dq = {ax.x * sh, ax.y * sh, ax.z * sh, ch};
            q = qmul(dq, q);
            const float inv = 1.0f / sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
            q.x *= inv; q.y *= inv; q.z *= inv; q.w *= inv;
        }
        s_R = qmatrix(q);
        s_cm = cm;
        a.rot[b] = make_float4(q.x, q.y, q.z, q.w);
        a.cm[b] = make_float4(cm.x, cm.y, cm.z, 0.f);
    }
    __syncthreads();
    const Mat3 R = s_R;
    const float3 cmv = s_cm;
    for (int t = threadIdx.x; t < np; t += kSmThreads) {
        const float3 q = f3(a.rest[rg.x + t]);
        const int id = to_new[rg.x + t];
        const float3 g = ((R.c0 * q.x + R.c1 * q.y) + R.c2 * q.z) + cmv;
        const float4 p4 = P[id];
        P[id] = make_float4(g.x, g.y, g.z, p4.w);
        track_displacement(C, id, g, true);
    }
}

void launch_shape_matching(cudaStream_t st, const SimConsts &C, const RigidArgs &a, float4 *P,
                           const int *to_new, LaunchLog *L)
{
    if (a.num_bodies <= 0) return;
    k_shape_matching<<<a.num_bodies, kSmThreads, 0, st>>>(C, a, P, to_new);
    L->done(__func__);
}

__global__ void k_immovable(SimConsts C, int k, const int *__restrict__ ids, const int *__restrict__ to_new,
                            const float4 *__restrict__ Xs, float4 *__restrict__ P)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= k) return;
    const int i = to_new[ids[t]];
    const float4 x = Xs[i];
    P[i] = make_float4(x.x, x.y, x.z, P[i].w);
    track_displacement(C, i, f3(x), true);
}

void launch_immovable(cudaStream_t st, const SimConsts &C, int k, const int *ids, const int *to_new,
                      const float4 *Xs, float4 *P, LaunchLog *L)
{
    if (k <= 0) return;
    k_immovable<<<(k + 255) / 256, 256, 0, st>>>(C, k, ids, to_new, Xs, P);
    L->done(__func__);
}

// setParticle (particlesolver.cuh:388-393) on the picked particle.
__global__ void k_pick(int id_orig, const int *__restrict__ to_new, float4 *pos, float3 p, int set_pos, float4 *vel,
                       float3 v)
{
    const int i = to_new[id_orig];
    if (set_pos) {
        const float4 o = pos[i];
        pos[i] = make_float4(p.x, p.y, p.z, o.w);
    }
    if (vel) {
        const float4 o = vel[i];
        vel[i] = make_float4(v.x, v.y, v.z, o.w);
    }
}

void launch_pick(cudaStream_t st, int id_orig, const int *to_new, float4 *pos, float3 p, int set_pos, float4 *vel,
                 float3 v, LaunchLog *L)
{
    k_pick<<<1, 1, 0, st>>>(id_orig, to_new, pos, p, set_pos, vel, v);
    L->done(__func__);
}

// {x, y, z, phase} records for a renderer.
__global__ void k_pack_infos(int n, const float4 *__restrict__ X, const float4 *__restrict__ V, float4 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = X[i];
    out[i] = make_float4(x.x, x.y, x.z, V[i].w);
}

void launch_pack_infos(cudaStream_t st, int n, const float4 *X, const float4 *V, void *out)
{
    if (n <= 0) return;
    k_pack_infos<<<(n + 255) / 256, 256, 0, st>>>(n, X, V, (float4 *)out);
}

__global__ void k_gather_xyz(int n, const float4 *__restrict__ src, const int *__restrict__ map,
                             float *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = src[i];
    const int o = map ? map[i] : i;
    out[3 * o] = v.x;
    out[3 * o + 1] = v.y;
    out[3 * o + 2] = v.z;
}

void launch_gather_xyz(cudaStream_t st, int n, const float4 *src, const int *map, float *out)
{
    if (n <= 0) return;
    k_gather_xyz<<<(n + 255) / 256, 256, 0, st>>>(n, src, map, out);
}

__global__ void k_scatter_xyz(int n, const float *__restrict__ in, const int *__restrict__ map,
                              float4 *__restrict__ dst)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = map ? map[k] : k;
    const float4 o = dst[i];
    dst[i] = make_float4(in[3 * k], in[3 * k + 1], in[3 * k + 2], o.w);
}

void launch_scatter_xyz(cudaStream_t st, int n, const float *in, const int *map, float4 *dst)
{
    if (n <= 0) return;
    k_scatter_xyz<<<(n + 255) / 256, 256, 0, st>>>(n, in, map, dst);
}

// Device error word: NaN / Inf positions.
__global__ void k_check_finite(int n, const float4 *__restrict__ X, unsigned *err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = X[i];
    const bool bad = !(isfinite(x.x) && isfinite(x.y) && isfinite(x.z));
    if (__any_sync(__activemask(), bad) && bad) atomicOr(err, BP_DEVERR_NONFINITE);
}

void launch_check_finite(cudaStream_t st, int n, const float4 *X, unsigned *err, LaunchLog *L)
{
    if (n <= 0) return;
    k_check_finite<<<(n + 255) / 256, 256, 0, st>>>(n, X, err);
    L->done(__func__);
}

}  // namespace bp
