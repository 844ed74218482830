// bp_grid.cu -- hash grid: cell keys, stable radix sort, cell ranges, reorder.
//
// Replaces updateGrid() of the reference (brasstower/particlesolver.cuh:712-765):
//   updateGridId        (kernel/grid.cuh:30-47)   -> k_hash_*  (+ fused pass-0 histogram)
//   cub::DeviceRadixSort::SortPairs (PS:721-738) -> own LSD radix sort, 9-bit digits
//   findStartEndId      (kernel/grid.cuh:70-99)   -> k_find_start_end (stand-alone API)
//                                                    k_cell_offsets (dense prefix, solver)
//   reorderParticlesData (kernel/grid.cuh:134-163)
//   + inverseMapping    (kernel/util.cuh:348-358) -> k_reorder (float4 records, fused predict,
//                                                    mass scaling and plane stabilisation)
#include <algorithm>

#include "bp_internal.h"

namespace bp {

// ------------------------------------------------------------------------
// radix sort
// ------------------------------------------------------------------------

size_t sort_scratch_bytes(int n, int D)
{
    const size_t tiles = (size_t)sort_tiles(n);
    const int passes = sort_passes(D);
    const size_t alts = passes > 2 ? 2 : 1;
    size_t b = alts * 2 * ((size_t)n * 4 + 256);
    b += (size_t)kRadixBins * tiles * 4 + 256;
    b += (size_t)kRadixBins * 4 + 256;
    return b;
}

void sort_scratch_carve(void *base, int n, int D, SortScratch *s)
{
    char *p = (char *)base;
    auto take = [&](size_t bytes) {
        char *r = p;
        p += (bytes + 255) & ~(size_t)255;
        return r;
    };
    const int passes = sort_passes(D);
    const size_t tiles = (size_t)sort_tiles(n);
    s->keys_alt[0] = (int *)take((size_t)n * 4);
    s->vals_alt[0] = (int *)take((size_t)n * 4);
    if (passes > 2) {
        s->keys_alt[1] = (int *)take((size_t)n * 4);
        s->vals_alt[1] = (int *)take((size_t)n * 4);
    } else {
        s->keys_alt[1] = s->keys_alt[0];
        s->vals_alt[1] = s->vals_alt[0];
    }
    s->hist = (int *)take((size_t)kRadixBins * tiles * 4);
    s->digit_total = (int *)take((size_t)kRadixBins * 4);
}

// Per-tile digit histogram, digit-major: hist[d * tiles + tile].
__global__ void __launch_bounds__(kSortThreads) k_radix_upsweep(const int *__restrict__ keys, int n, int shift,
                                                               int *__restrict__ hist, int tiles, Gate gate)
{
    if (gate_closed(gate)) return;
    __shared__ int h[kRadixBins];
    for (int d = threadIdx.x; d < kRadixBins; d += kSortThreads) h[d] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const int idx = base + k * kSortThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & (kRadixBins - 1)], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadixBins; d += kSortThreads) hist[(size_t)d * tiles + blockIdx.x] = h[d];
}

// One CTA per digit: exclusive scan over the tiles, digit total on the side.
__global__ void __launch_bounds__(256) k_radix_scan(int *__restrict__ hist, int tiles, int *__restrict__ digit_total,
                                                    Gate gate)
{
    if (gate_closed(gate)) return;
    __shared__ int warp_sums[8];
    int *row = hist + (size_t)blockIdx.x * tiles;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int carry = 0;
    for (int base = 0; base < tiles; base += 256) {
        const int idx = base + threadIdx.x;
        const int v = idx < tiles ? row[idx] : 0;
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            int ws = lane < 8 ? warp_sums[lane] : 0;
#pragma unroll
            for (int o = 1; o < 8; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, ws, o);
                if (lane >= o) ws += t;
            }
            if (lane < 8) warp_sums[lane] = ws;  // inclusive over warps
        }
        __syncthreads();
        const int warp_prefix = warp ? warp_sums[warp - 1] : 0;
        if (idx < tiles) row[idx] = carry + warp_prefix + incl - v;
        const int chunk_total = warp_sums[7];
        __syncthreads();
        carry += chunk_total;
    }
    if (threadIdx.x == 0) digit_total[blockIdx.x] = carry;
}

// Stable scatter of one tile.  Each warp owns a contiguous 256-key segment
// (8 rounds of 32); within a round lanes holding the same digit are ranked
// with __match_any_sync, so the order inside the tile is preserved: warp
// segment first, then round, then lane.
__global__ void __launch_bounds__(kSortThreads) k_radix_downsweep(
    const int *__restrict__ keys_in, const int *__restrict__ vals_in, int n, int shift,
    const int *__restrict__ hist, const int *__restrict__ digit_total, int tiles, int *__restrict__ keys_out,
    int *__restrict__ vals_out, Gate gate)
{
    if (gate_closed(gate)) return;
    constexpr int W = kSortThreads / 32;
    constexpr int SEG = kSortTile / W;        // keys per warp
    constexpr int ROUNDS = SEG / 32;
    __shared__ int cnt[W][kRadixBins];
    __shared__ int dbase[kRadixBins];
    __shared__ int wsum[W];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int e = threadIdx.x; e < W * kRadixBins; e += kSortThreads) (&cnt[0][0])[e] = 0;

    // exclusive prefix of the digit totals (one digit per thread)
    {
        const int d = threadIdx.x;  // kSortThreads == kRadixBins
        const int v = digit_total[d];
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        int wp = 0;
        for (int k = 0; k < warp; ++k) wp += wsum[k];
        dbase[d] = wp + incl - v + hist[(size_t)d * tiles + blockIdx.x];
    }
    __syncthreads();

    int key[ROUNDS], val[ROUNDS], dig[ROUNDS], loc[ROUNDS];
    const int seg0 = blockIdx.x * kSortTile + warp * SEG;
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
        const int idx = seg0 + r * 32 + lane;
        const bool valid = idx < n;
        key[r] = valid ? keys_in[idx] : 0;
        val[r] = valid ? (vals_in ? vals_in[idx] : idx) : 0;
        const int d = valid ? ((key[r] >> shift) & (kRadixBins - 1)) : kRadixBins;
        dig[r] = d;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int before = __popc(peers & lt);
        int base = 0;
        if (valid) base = cnt[warp][d];
        __syncwarp();
        if (valid && before == 0) cnt[warp][d] = base + __popc(peers);
        __syncwarp();
        loc[r] = base + before;
    }
    __syncthreads();
    {
        const int d = threadIdx.x;
        int run = 0;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const int c = cnt[w][d];
            cnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
        const int idx = seg0 + r * 32 + lane;
        if (idx < n) {
            const int pos = dbase[dig[r]] + cnt[warp][dig[r]] + loc[r];
            keys_out[pos] = key[r];
            vals_out[pos] = val[r];
        }
    }
}

void radix_sort_pairs(cudaStream_t st, int n, int D, const int *keys_in, const int *vals_in, int *keys_out,
                      int *vals_out, const SortScratch &s, bool hist_ready, LaunchLog *L, Gate gate)
{
    if (n <= 0) return;
    const int tiles = sort_tiles(n);
    const int passes = sort_passes(D);
    const int *ksrc = keys_in, *vsrc = vals_in;
    for (int p = 0; p < passes; ++p) {
        const int shift = p * kRadixBits;
        int *kdst = (p == passes - 1) ? keys_out : s.keys_alt[p & 1];
        int *vdst = (p == passes - 1) ? vals_out : s.vals_alt[p & 1];
        if (!(p == 0 && hist_ready)) {
            k_radix_upsweep<<<tiles, kSortThreads, 0, st>>>(ksrc, n, shift, s.hist, tiles, gate);
            L->done("k_radix_upsweep");
        }
        k_radix_scan<<<kRadixBins, 256, 0, st>>>(s.hist, tiles, s.digit_total, gate);
        L->done("k_radix_scan");
        k_radix_downsweep<<<tiles, kSortThreads, 0, st>>>(ksrc, vsrc, n, shift, s.hist, s.digit_total, tiles,
                                                          kdst, vdst, gate);
        L->done("k_radix_downsweep");
        ksrc = kdst;
        vsrc = vdst;
    }
}

// ------------------------------------------------------------------------
// cell keys
// ------------------------------------------------------------------------

// Tile layout identical to the sort (4096 keys per CTA) so the pass-0
// histogram is produced here and the first upsweep is skipped.
template <class Key>
__device__ __forceinline__ void hash_tile(int n, Key key_of, int *__restrict__ keys, int *__restrict__ hist, int tiles)
{
    __shared__ int h[kRadixBins];
    for (int d = threadIdx.x; d < kRadixBins; d += kSortThreads) h[d] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const int idx = base + k * kSortThreads + threadIdx.x;
        if (idx < n) {
            const int key = key_of(idx);
            keys[idx] = key;
            atomicAdd(&h[key & (kRadixBins - 1)], 1);
        }
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadixBins; d += kSortThreads) hist[(size_t)d * tiles + blockIdx.x] = h[d];
}

__device__ __forceinline__ int hash_key(float3 p, float cell, int D, unsigned m)
{
    return cell_addr(cell_coord(p.x, cell), cell_coord(p.y, cell), cell_coord(p.z, cell), D, m);
}

__global__ void __launch_bounds__(kSortThreads) k_hash_f3(int n, const float *__restrict__ pos3, float cell, int D,
                                                          int *__restrict__ keys, int *__restrict__ hist, int tiles)
{
    const unsigned m = (unsigned)D - 1u;
    hash_tile(
        n,
        [&](int i) { return hash_key(make_float3(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]), cell, D, m); },
        keys, hist, tiles);
}

// predictPositions + applyGravity (PS:59-69, 49-57) feeding the hash; the
// rounding is pinned (no fused multiply-add) so that the prediction, and with
// it every cell key, is bit-identical to a host evaluation of x + v*dt + (g*dt)*dt.
__device__ __forceinline__ float3 predict(float3 x, float3 v, float3 gr, const SimConsts &C)
{
    float3 p;
    p.x = __fadd_rn(x.x, __fmul_rn(v.x, C.dt));
    p.y = __fadd_rn(x.y, __fmul_rn(v.y, C.dt));
    p.z = __fadd_rn(x.z, __fmul_rn(v.z, C.dt));
    p.x = __fadd_rn(p.x, __fmul_rn(__fmul_rn(gr.x, C.dt), C.dt));
    p.y = __fadd_rn(p.y, __fmul_rn(__fmul_rn(gr.y, C.dt), C.dt));
    p.z = __fadd_rn(p.z, __fmul_rn(__fmul_rn(gr.z, C.dt), C.dt));
    return p;
}

// Cell key of the predicted position; in a batched ensemble the key of the
// particle's scene grid, offset by the scene's first key.  Every particle of
// a scene keeps its scene's index segment, so X/V index i has scene_of[i].
__global__ void __launch_bounds__(kSortThreads) k_hash_state(SimConsts C, const float4 *__restrict__ X,
                                                             const float4 *__restrict__ V, int *__restrict__ keys,
                                                             int *__restrict__ hist, int tiles)
{
    hash_tile(
        C.n,
        [&](int i) {
            const int s = scene_index(C, i);
            const float3 p = predict(f3(X[i]), f3(V[i]), gravity_of(C, s), C);
            if (s < 0) return hash_key(p, C.cell, C.D, C.mask);
            const SceneConsts &S = C.scn[s];
            return S.base + hash_key(p, C.cell, S.D, S.mask);
        },
        keys, hist, tiles);
}

void launch_hash_f3(cudaStream_t st, int n, const float *pos3, float cell, int D, int *keys, int *hist,
                    LaunchLog *L)
{
    if (n <= 0) return;
    const int tiles = sort_tiles(n);
    k_hash_f3<<<tiles, kSortThreads, 0, st>>>(n, pos3, cell, D, keys, hist, tiles);
    L->done(__func__);
}

void launch_hash_state(cudaStream_t st, const SimConsts &C, const float4 *X, const float4 *V, int *keys,
                       int *hist, LaunchLog *L)
{
    if (C.n <= 0) return;
    const int tiles = sort_tiles(C.n);
    k_hash_state<<<tiles, kSortThreads, 0, st>>>(C, X, V, keys, hist, tiles);
    L->done(__func__);
}

// ------------------------------------------------------------------------
// cell ranges
// ------------------------------------------------------------------------

// findStartEndId semantics (kernel/grid.cuh:70-99): only occupied cells are written.
__global__ void k_find_start_end(int n, const int *__restrict__ sorted, int *__restrict__ start,
                                 int *__restrict__ end)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int u = sorted[i];
    if (i == 0 || sorted[i - 1] != u) start[u] = i;
    if (i == n - 1 || sorted[i + 1] != u) end[u] = i + 1;
}

// resetStartEndId semantics (kernel/grid.cuh:101-132).
__global__ void k_reset_start_end(int n, const int *__restrict__ sorted, int *__restrict__ start,
                                  int *__restrict__ end)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int u = sorted[i];
    if (i == 0 || sorted[i - 1] != u) start[u] = -1;
    if (i == n - 1 || sorted[i + 1] != u) end[u] = -1;
}

// Dense prefix: off[c] = number of particles whose key is below c, for
// c in [0, ncells].  Dense or small tables (per == 1): one cell per thread,
// found by a binary search over all keys.  Large tables with many more cells
// than particles (mostly empty cells) give each warp 32 * per consecutive cells:
// lanes 0 and 31 search the keys at the ends of that range, the warp copies
// the keys between them into shared memory, and lane l takes cells l,
// l + 32, l + 64, ... of the range (so that every store of the warp writes
// 32 consecutive entries), counting the copied keys below each cell from
// where its previous cell's count stopped.  A range holding more keys than
// the copy takes searches among them instead.
constexpr int kOffsetKeysPerWarp = 512;

__device__ __forceinline__ int lower_bound_key(const int *__restrict__ sorted, int lo, int hi, long long c)
{
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(sorted + mid) < c) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(256) k_cell_offsets(int n, int ncells, int per, const int *__restrict__ sorted,
                                                      int *__restrict__ off, Gate gate)
{
    __shared__ int keys[256 / 32][kOffsetKeysPerWarp];
    if (gate_closed(gate)) return;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (per == 1) {
        if (t <= ncells) off[t] = lower_bound_key(sorted, 0, n, t);
        return;
    }
    const int lane = threadIdx.x & 31;
    int *wk = keys[threadIdx.x >> 5];
    const long long w0 = (t - lane) * per, w1 = w0 + 32LL * per;  // the warp's cells [w0, w1)
    int a = 0, b = n;
    if (lane == 0) a = lower_bound_key(sorted, 0, n, w0);
    if (lane == 31) b = lower_bound_key(sorted, 0, n, w1);
    a = __shfl_sync(0xffffffffu, a, 0);
    b = __shfl_sync(0xffffffffu, b, 31);
    // every key before a is below w0, the key at b (if any) is at least w1
    const int cnt = b - a;
    if (cnt <= kOffsetKeysPerWarp) {
        for (int q = lane; q < cnt; q += 32) wk[q] = __ldg(sorted + a + q);
        __syncwarp();
        int lo = 0;
        for (long long c = w0 + lane; c < w1 && c <= ncells; c += 32) {
            while (lo < cnt && wk[lo] < c) ++lo;
            off[c] = a + lo;
        }
    } else {
        int lo = a;
        for (long long c = w0 + lane; c < w1 && c <= ncells; c += 32) {
            lo = lower_bound_key(sorted, lo, b, c);
            off[c] = lo;
        }
    }
}

void launch_find_start_end(cudaStream_t st, int n, const int *sorted, int *start, int *end, LaunchLog *L)
{
    if (n <= 0) return;
    k_find_start_end<<<(n + 255) / 256, 256, 0, st>>>(n, sorted, start, end);
    L->done(__func__);
}

void launch_reset_start_end(cudaStream_t st, int n, const int *sorted, int *start, int *end, LaunchLog *L)
{
    if (n <= 0) return;
    k_reset_start_end<<<(n + 255) / 256, 256, 0, st>>>(n, sorted, start, end);
    L->done(__func__);
}

void launch_cell_offsets(cudaStream_t st, int n, int ncells, const int *sorted, int *off, LaunchLog *L, Gate gate)
{
    // the warp ranges pay on large sparse tables; a smaller table takes a
    // thread per cell, which fills the GPU (32k particles on a 64^3 table:
    // 0.081 ms per frame with warp ranges, 0.052 with a search per 8 cells)
    const int per = (ncells > 4LL * n && ncells >= (1 << 22)) ? 32 : 1;
    const long long threads = ((long long)ncells + 1 + per - 1) / per;
    k_cell_offsets<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(n, ncells, per, sorted, off, gate);
    L->done(__func__);
}

// ------------------------------------------------------------------------
// reorder
// ------------------------------------------------------------------------

// Gathers the float4 records into cell order, recomputes the prediction
// (bit-identical to the hashed one), then computeInvScaledMasses (PS:84-98,
// on x before stabilisation), two rounds of planeStabilize (PS:822-833) and,
// when nothing else runs between, iteration 0's plane collision.
__global__ void __launch_bounds__(256) k_reorder(SimConsts C, ReorderArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C.n) return;
    const int o = a.order[i];
    const float4 X = a.Xc[o];
    const float4 V = a.Vc[o];
    const int id = a.orig_c[o];
    const int s = scene_index(C, i);
    float3 x = f3(X), v = f3(V);
    float3 p = predict(x, v, gravity_of(C, s), C);
    if (a.cls) {  // the hashed position: its real cell gives the class
        const int3 c = cell_of(p, C);
        a.cls[i] = alias_class(c.x, c.y, c.z, s < 0 ? C.D : C.scn[s].D);
        a.pos0[i] = make_float4(p.x, p.y, p.z, 0.f);
    }
    if (a.hash_pos) a.hash_pos[i] = make_float4(p.x, p.y, p.z, 0.f);  // the position its cell was hashed from
    if (a.inv_scaled) {
        const float scale = powf(2.7182818284f, -C.mass_k * x.y);
        a.inv_scaled[i] = 1.0f / (scale * X.w);
    }
    if (a.stabilize) {
        plane_stabilize(C, s, x, p);
        plane_stabilize(C, s, x, p);
    }
    if (a.collide) plane_collide(C, s, x, p);
    a.Xs[i] = make_float4(x.x, x.y, x.z, X.w);
    a.Vs[i] = V;
    if (a.tile_solid && phase_of(V) > 0) a.tile_solid[i >> 8] = 1;
    a.P[i] = make_float4(p.x, p.y, p.z, V.w);
    a.mass[i] = X.w;
    a.orig_s[i] = id;
    a.to_new[id] = i;
}

void launch_reorder(cudaStream_t st, const SimConsts &C, const ReorderArgs &a, LaunchLog *L)
{
    if (C.n <= 0) return;
    k_reorder<<<(C.n + 255) / 256, 256, 0, st>>>(C, a);
    L->done(__func__);
}

// ------------------------------------------------------------------------
// alias classes
// ------------------------------------------------------------------------

// Counts the particles whose class differs from their cell's first
// particle's (about how many candidates the class walks would skip) and
// opens the substep's classes (*moved = 0).
__global__ void __launch_bounds__(256) k_class_count(int n, const int *__restrict__ sorted_keys,
                                                     const int *__restrict__ off, ClassArrays a)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j == 0) *a.moved = 0;
    bool differs = false;
    if (j < n) differs = __ldg(a.cls + j) != __ldg(a.cls + __ldg(off + __ldg(sorted_keys + j)));
    const unsigned votes = __ballot_sync(0xffffffffu, differs);
    if ((threadIdx.x & 31) == 0 && votes) atomicAdd(a.mixed, __popc(votes));
}

// keys[q] holds the class of perm[q] on entry (the radix pass output).
__global__ void __launch_bounds__(256) k_class_keys(int n, const int *__restrict__ sorted_keys,
                                                    const float *__restrict__ mass, ClassArrays a, Gate gate)
{
    if (gate_closed(gate)) return;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int j = a.perm[q];
    a.keys[q] = a.keys[q] * a.T + __ldg(sorted_keys + j);
    a.inv[j] = q;
    a.mass[q] = __ldg(mass + j);
}

static Gate class_gate(int n, const ClassArrays &a) { return Gate{a.mixed, (n + 31) / 32}; }

void launch_class_order(cudaStream_t st, int n, const int *sorted_keys, const int *off, const float *mass,
                        const ClassArrays &a, const SortScratch &s, LaunchLog *L)
{
    if (n <= 0) return;
    cudaMemsetAsync(a.mixed, 0, sizeof(int), st);
    k_class_count<<<(n + 255) / 256, 256, 0, st>>>(n, sorted_keys, off, a);
    L->done("k_class_count");
    // the rest runs only where the classes pay (see k_class_refresh)
    const Gate gate = class_gate(n, a);
    // one 9-bit digit covers the 3 class bits: a stable partition of the sorted order
    radix_sort_pairs(st, n, 8, a.cls, nullptr, a.keys, a.perm, s, false, L, gate);
    k_class_keys<<<(n + 255) / 256, 256, 0, st>>>(n, sorted_keys, mass, a, gate);
    L->done("k_class_keys");
    launch_cell_offsets(st, n, 8 * a.T, a.keys, a.off, L, gate);
}

// Writes particle p's x, y, z and phase bits to slot q of the walk planes
// (SimConsts::walk_xyz).
__device__ __forceinline__ void put_planes(float *planes, int stride, int q, float4 p)
{
    const size_t st = (size_t)stride;
    planes[q] = p.x;
    planes[st + q] = p.y;
    planes[2 * st + q] = p.z;
    planes[3 * st + q] = p.w;
}

// Walks use the classes while at least 1/32 of the particles sit in a cell
// holding another class (below that the extra indirection costs more than
// the skipped candidates save) and no particle has left the reach.
// *moved: 1 where the gate is closed, 2 where a particle left the reach.
// planes != nullptr: also writes the walk planes, in sorted order where the
// gate is closed and in class order where it is open.
__global__ void __launch_bounds__(256) k_class_refresh(int n, const float4 *__restrict__ P,
                                                       const float4 *__restrict__ V, ClassArrays a, Gate gate,
                                                       float *__restrict__ planes, int stride)
{
    if (gate_closed(gate)) {  // uniform: written by an earlier kernel
        if (blockIdx.x == 0 && threadIdx.x == 0) *a.moved = 1;
        if (planes)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
                put_planes(planes, stride, i, P[i]);
        return;
    }
    bool far = false;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int j = __ldg(a.perm + q);
        const float4 p = P[j];
        a.pos[q] = p;
        if (planes) put_planes(planes, stride, q, p);
        if (V) a.vel[q] = V[j];
        const float4 p0 = __ldg(a.pos0 + j);
        const float dx = p.x - p0.x, dy = p.y - p0.y, dz = p.z - p0.z;
        // NaN counts as moved; so do positions far enough out that the hash's
        // float rounding exceeds the reach's margin
        const bool inside = fabsf(p.x) < 4.0e4f && fabsf(p.y) < 4.0e4f && fabsf(p.z) < 4.0e4f;
        far |= !(dx * dx + dy * dy + dz * dz <= a.reach2) || !inside;
    }
    if (far) *a.moved = 2;
}

// Blocks of a grid-stride loop over one resident wave (8 CTAs of 256 per SM).
static int wave_blocks(int n)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return std::min((n + 255) / 256, std::max(sms, 1) * 8);
}

void launch_class_refresh(cudaStream_t st, int n, const float4 *P, const ClassArrays &a, LaunchLog *L,
                          const float4 *V, float *planes, int stride)
{
    if (n <= 0) return;
    // the common case without planes is the gate's early exit (one wave);
    // with planes, a thread per particle
    const int blocks = planes ? (n + 255) / 256 : wave_blocks(n);
    k_class_refresh<<<blocks, 256, 0, st>>>(n, P, V, a, class_gate(n, a), planes, stride);
    L->done(__func__);
}

// The walk planes in sorted order (scenes without alias classes).
__global__ void __launch_bounds__(256) k_walk_planes(int n, const float4 *__restrict__ P, float *__restrict__ planes,
                                                     int stride)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        put_planes(planes, stride, i, P[i]);
}

void launch_walk_planes(cudaStream_t st, int n, const float4 *P, float *planes, int stride, LaunchLog *L)
{
    if (n <= 0) return;
    k_walk_planes<<<(n + 255) / 256, 256, 0, st>>>(n, P, planes, stride);
    L->done(__func__);
}

}  // namespace bp
