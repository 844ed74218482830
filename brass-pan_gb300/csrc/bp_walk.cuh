// bp_walk.cuh -- neighbour walks of the scan kernels, staged in shared memory.
//
// A CTA of kWalkThreads threads handles kWalkThreads consecutive particles of
// the cell-sorted arrays.  Because cells are addressed x-major, those
// particles lie in one or two (x, y) columns of the grid, over a run of z
// cells; the 27-cell neighbourhoods of all of them are covered by at most 9
// column runs per column (split in two where z wraps around the table).
// stage_block() copies those runs of P into shared memory with coalesced
// loads; every candidate read of the walk then comes from shared memory.
// A CTA whose runs would not fit (three or more columns, or more than
// kStageCap particles) and particles that left their stored cell read P from
// global memory instead.
//
// Every walk visits the candidates of the 27 cells column by column, in
// ascending sorted index within a column, or the subset of them recorded in
// the particle's Verlet list (see SimConsts::vl); the pair sums of the scan
// kernels therefore accumulate in the same order on every path.
//
// A walk takes two functions: test(j, pj), the cheap pair filter (distance,
// phases), and body(j, pj), the pair term.  Split walks first test a chunk of
// up to 32 candidates into a bit mask and then run the body over the set
// bits only, so a warp issues the body about as often as its busiest lane
// has neighbours, instead of once per candidate of the longest run.
//
// In a batched ensemble the walk uses the grid of the particle's own scene
// (GridView); a CTA whose particles belong to two scenes is not staged.
#pragma once

#include "bp_common.cuh"

namespace bp {

constexpr int kWalkThreads = 256;
// Staged particles per CTA (44 KB at 2816) and the CTAs per SM the scan
// kernels are compiled for (registers per thread <= 65536 / (256 x that)).
// Four CTAs (64 registers) measured 7 % faster on the mixed scene than the
// three that the lambda and pass A kernels fall to at their natural 66-71
// registers; five spill.
#ifndef BP_STAGE_CAP
#define BP_STAGE_CAP 2816
#endif
#ifndef BP_SCAN_MIN_BLOCKS
#define BP_SCAN_MIN_BLOCKS 4
#endif
// Candidate tests a split walk unrolls (loads in flight per thread).
#ifndef BP_CHUNK_UNROLL
#define BP_CHUNK_UNROLL 4
#endif
constexpr int kChunkUnroll = BP_CHUNK_UNROLL;
// Candidate tests of a chunk gathered four at a time into a nibble of
// constant bit positions, then shifted into the chunk mask once (measured on
// the mixed scene against one variable shift per candidate: lambda 5.73 ->
// 5.60 ms per frame early, 6.96 -> 6.73 late; the step 222.0 -> 225.2 M and
// 133.5 -> 137.3 M particle-substeps/s).  0 keeps the per-candidate form.
#ifndef BP_CHUNK_NIBBLES
#define BP_CHUNK_NIBBLES 1
#endif

// The test bits of candidates [0, cnt) of a chunk read from s: bit t set when
// test(t, s[t]) holds (t is the candidate's offset in the chunk).
template <class F>
__device__ __forceinline__ unsigned chunk_bits(int cnt, const float4 *s, F &&test)
{
    unsigned bits = 0u;
#if BP_CHUNK_NIBBLES
    int t = 0;
#pragma unroll 1
    for (; t + 4 <= cnt; t += 4) {
        const float4 a = s[t], b = s[t + 1], c = s[t + 2], d = s[t + 3];
        const unsigned nib = (test(t, a) ? 1u : 0u) | (test(t + 1, b) ? 2u : 0u) | (test(t + 2, c) ? 4u : 0u) |
                             (test(t + 3, d) ? 8u : 0u);
        bits |= nib << t;
    }
#pragma unroll 1
    for (; t < cnt; ++t)
        if (test(t, s[t])) bits |= 1u << t;
#else
#pragma unroll kChunkUnroll
    for (int t = 0; t < cnt; ++t)
        if (test(t, s[t])) bits |= 1u << t;
#endif
    return bits;
}
constexpr int kStageCap = BP_STAGE_CAP;
constexpr int kStageSegs = 2 * 9 * 2; // groups x columns x pieces

struct StageShared {
    float4 pos[kStageCap];
    int gstart[kStageSegs];
    int len[kStageSegs];
    int sbase[kStageSegs];
    int keys[kWalkThreads];
    int first1;  // first thread of the second column group
    int ngroups;
    int ok;
    int scene;
    int has_solid;  // a solid lies in the CTA's runs (tile_solid) or among the staged particles
};

constexpr int kNoSolidNear = -2;

// The staging buffer lives in dynamic shared memory, sized stage_bytes(C) at
// launch: without staging the kernels take none, and the L1 cache keeps the
// whole unified shared-memory / L1 array.
extern __shared__ __align__(16) unsigned char bp_stage_smem[];
__device__ __forceinline__ StageShared &stage_shared() { return *reinterpret_cast<StageShared *>(bp_stage_smem); }
inline size_t stage_bytes(const SimConsts &C) { return C.stage ? sizeof(StageShared) : 0; }

// Collective: every thread of the CTA must call it (before any early exit).
// Returns the calling thread's column group (0 or 1), or -1 when the CTA does
// not use shared memory or the thread has no particle.
//
// With `tile_solid` (one flag per 256 sorted particles: the tile holds a
// solid), a CTA of fluid particles whose runs touch no solid tile skips the
// staging and returns kNoSolidNear to every thread: none of its particles
// that stayed in their stored cell can meet a solid.
//
// With copy == false only the runs and the solid check are made: the CTA
// walks nothing from shared memory (the returned group is -1 or kNoSolidNear).
__device__ __forceinline__ int stage_block(const SimConsts &C, const float4 *__restrict__ P,
                                           const int *__restrict__ off_all, int i0, StageShared &S,
                                           const int *__restrict__ tile_solid = nullptr, bool copy = true)
{
    if (!C.stage) return -1;  // uniform across the grid: no barrier skipped unevenly
    const int t = threadIdx.x;
    const int i = i0 + t;
    const bool valid = i < C.n;
    if (t == 0) {
        S.scene = scene_index(C, i0);
        S.first1 = kWalkThreads;
        S.has_solid = 0;
    }
    __syncthreads();
    const int s0 = S.scene;
    if (!__syncthreads_and(!valid || scene_index(C, i) == s0)) return -1;
    const GridView v = grid_view(C, s0, off_all);
    const unsigned D = (unsigned)v.D, m = v.mask;
    const int key = valid ? __ldg(C.cell_keys + i) - v.base : -1;
    S.keys[t] = key;
    __syncthreads();
    const bool boundary = valid && (t == 0 || (unsigned)key / D != (unsigned)S.keys[t - 1] / D);
    const int G = __syncthreads_count(boundary);
    if (boundary && t > 0) S.first1 = t;  // unique when G == 2
    __syncthreads();
    if (G < 1 || G > 2) return -1;
    const int nvalid = min(kWalkThreads, C.n - i0);
    if (t < G * 9) {
        const int g = t / 9, k = t % 9;
        const int tf = g == 0 ? 0 : S.first1;
        const int tl = g == G - 1 ? nvalid - 1 : S.first1 - 1;
        const unsigned kf = (unsigned)S.keys[tf], kl = (unsigned)S.keys[tl];
        const unsigned colid = kf / D;
        const unsigned x = colid / D, y = colid % D;
        const int zlo = (int)(kf % D) - 1, zhi = (int)(kl % D) + 1;
        const unsigned nx = (x + (unsigned)(k / 3) - 1u) & m, ny = (y + (unsigned)(k % 3) - 1u) & m;
        const unsigned base = (nx * D + ny) * D;
        const int a = max(zlo, 0), b = min(zhi, (int)D - 1);
        const int sa = __ldg(v.off + base + a), ea = __ldg(v.off + base + b + 1);
        int sb = 0, eb = 0;
        if (zlo < 0 && zhi <= (int)D - 1) {  // wraps below: cell D-1
            sb = __ldg(v.off + base + D - 1);
            eb = __ldg(v.off + base + D);
        } else if (zhi > (int)D - 1 && zlo >= 0) {  // wraps above: cell 0
            sb = __ldg(v.off + base);
            eb = __ldg(v.off + base + 1);
        }
        S.gstart[2 * t] = sa;
        S.len[2 * t] = ea - sa;
        S.gstart[2 * t + 1] = sb;
        S.len[2 * t + 1] = eb - sb;
        if (tile_solid) {
            bool solid = false;
            for (int q = sa >> 8; q <= (ea - 1) >> 8 && ea > sa && !solid; ++q) solid = __ldg(tile_solid + q) != 0;
            for (int q = sb >> 8; q <= (eb - 1) >> 8 && eb > sb && !solid; ++q) solid = __ldg(tile_solid + q) != 0;
            if (solid) S.has_solid = 1;
        }
    }
    if (tile_solid) {
        const bool own_solid = valid && phase_of(P[i]) > 0;
        // uniform: S.has_solid was written before the barrier
        if (!__syncthreads_or(own_solid) && !S.has_solid) return kNoSolidNear;
    }
    __syncthreads();
    if (t == 0) {
        int total = 0;
        for (int s = 0; s < 2 * G * 9; ++s) {
            S.sbase[s] = total;
            total += S.len[s];
        }
        S.ok = total <= kStageCap;
        S.ngroups = G;
    }
    __syncthreads();
    if (!S.ok || !copy) return -1;
    bool solid = false;
    for (int s = 0; s < 2 * G * 9; ++s) {
        const int gs = S.gstart[s], l = S.len[s], sb = S.sbase[s];
        for (int u = t; u < l; u += kWalkThreads) {
            const float4 q = P[gs + u];
            solid |= phase_of(q) > 0;
            S.pos[sb + u] = q;
        }
    }
    if (solid) S.has_solid = 1;
    __syncthreads();
    if (!valid) return -1;
    return (G == 2 && t >= S.first1) ? 1 : 0;
}

// Launch of a neighbour-scan kernel over C.n particles: a staged launch takes
// one kWalkThreads CTA per tile (its staging is sized for that); an unstaged
// one C.scan_block threads per CTA, and with C.scan_persist no more CTAs than
// the GPU holds at once, each striding over the tiles (the kernels loop over
// tiles of blockDim.x particles from blockIdx.x on).
template <class... KArgs, class... Args>
inline void launch_scan(void (*kernel)(KArgs...), const SimConsts &C, size_t smem, cudaStream_t st, Args &&...args)
{
    const int block = C.stage ? kWalkThreads : C.scan_block;
    int grid = (C.n + block - 1) / block;
    if (!C.stage && C.scan_persist) {
        int per = 0, dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, smem);
        const int resident = (per > 0 ? per : 1) * (sms > 0 ? sms : 1);
        grid = grid < resident ? grid : resident;
    }
    kernel<<<grid, block, smem, st>>>(static_cast<Args &&>(args)...);
}

// The cells a ranged walk visits: offsets from the walker's cell, each axis
// a sub-range of -1..1 (the whole 27 cells: CellRange{}).  The cells are
// visited in the order of the full walk, so a walk over a sub-range meets its
// candidates in the same order as the full walk does.
struct CellRange {
    int lox = -1, hix = 1, loy = -1, hiy = 1, loz = -1, hiz = 1;
};

// Shared-memory index of candidate run [b, e) of column k for group g, or -1.
__device__ __forceinline__ int staged_index(const StageShared &S, int g, int k, int b, int e)
{
    const int s = 2 * (g * 9 + k);
    if (b >= S.gstart[s] && e <= S.gstart[s] + S.len[s]) return S.sbase[s] + (b - S.gstart[s]);
    if (b >= S.gstart[s + 1] && e <= S.gstart[s + 1] + S.len[s + 1]) return S.sbase[s + 1] + (b - S.gstart[s + 1]);
    return -1;
}

// The particle that thread t (< n) of an unstaged walking kernel takes:
// sorted particle t, or, while the walks use the alias classes, the t-th
// particle of class order.  A warp's particles then share one class, so
// their runs coincide instead of splitting between the classes interleaved
// in a table cell.  Each particle's own result does not depend on the thread.
__device__ __forceinline__ int walker_index(const SimConsts &C, int t)
{
    return classes_on(C) ? __ldg(C.cls_perm + t) : t;
}

// Does particle i walk its CTA's staged runs (it is still in its stored cell)?
__device__ __forceinline__ bool walks_staged(const SimConsts &C, const GridView &v, int i, int3 c,
                                             const StageShared *S, int g)
{
    return S != nullptr && g >= 0 && cell_addr(c.x, c.y, c.z, v.D, v.mask) + v.base == __ldg(C.cell_keys + i);
}

// Candidates [jb, e) of one run, read from src[j - b]: the test of each pair,
// then the body of those that pass, in ascending j.
template <bool Split, class T, class B>
__device__ __forceinline__ void walk_run(int jb, int b, int e, const float4 *src, T &test, B &body)
{
    if constexpr (!Split) {
#pragma unroll 1
        for (int j = jb; j < e; ++j) {
            const float4 pj = src[j - b];
            if (test(j, pj)) body(j, pj);
        }
    } else {
#pragma unroll 1
        for (int j0 = jb; j0 < e; j0 += 32) {
            const int cnt = min(32, e - j0);
            const float4 *s = src + (j0 - b);
            unsigned bits = chunk_bits(cnt, s, [&](int t, float4 p) { return test(j0 + t, p); });
#pragma unroll 1
            while (bits) {
                const int t = __ffs(bits) - 1;
                bits &= bits - 1u;
                body(j0 + t, s[t]);
            }
        }
    }
}

// A neighbour list in records of four (SimConsts::nbr, SimConsts::vl): entry
// k of particle i is base[((k / 4) * n + i) * 4 + k % 4].  The writer keeps
// the current record in registers and stores each full one with a single
// 16-byte store, so a warp writes whole records.
struct ListWriter {
    int4 *rec;      // record 0 of particle i; record r at rec[r * n]
    size_t stride;  // n
    int cap;        // a multiple of 4
    int cnt = 0;
    int4 buf = make_int4(0, 0, 0, 0);
    __device__ __forceinline__ ListWriter(int *base, int cap_, int n, int i)
        : rec(reinterpret_cast<int4 *>(base) + i), stride((size_t)n), cap(cap_) {}
    __device__ __forceinline__ void push(int j)
    {
        const int q = cnt & 3;
        buf.x = q == 0 ? j : buf.x;
        buf.y = q == 1 ? j : buf.y;
        buf.z = q == 2 ? j : buf.z;
        buf.w = q == 3 ? j : buf.w;
        if (q == 3 && cnt < cap) rec[(size_t)(cnt >> 2) * stride] = buf;
        ++cnt;
    }
    // Appends c0 + t for every set bit t of bits, in ascending t: singly up
    // to a record boundary, then whole records of four (no per-entry select),
    // then the rest singly.  The entries are those push() gives.
    __device__ __forceinline__ void push_bits(int c0, unsigned bits)
    {
#pragma unroll 1
        while (bits && (cnt & 3)) {
            push(c0 + __ffs(bits) - 1);
            bits &= bits - 1u;
        }
#pragma unroll 1
        while (__popc(bits) >= 4) {
            int4 r;
            r.x = c0 + __ffs(bits) - 1;
            bits &= bits - 1u;
            r.y = c0 + __ffs(bits) - 1;
            bits &= bits - 1u;
            r.z = c0 + __ffs(bits) - 1;
            bits &= bits - 1u;
            r.w = c0 + __ffs(bits) - 1;
            bits &= bits - 1u;
            if (cnt < cap) rec[(size_t)(cnt >> 2) * stride] = r;
            cnt += 4;
        }
#pragma unroll 1
        while (bits) {
            push(c0 + __ffs(bits) - 1);
            bits &= bits - 1u;
        }
    }
    // Writes the last partial record; returns the count to store (-1: overflow).
    __device__ __forceinline__ int finish()
    {
        if ((cnt & 3) && cnt < cap) rec[(size_t)(cnt >> 2) * stride] = buf;
        return cnt <= cap ? cnt : -1;
    }
};

// The cnt entries of particle i's list, in order: f(j, P[j]).  Each record's
// four indices come in one 16-byte load and their positions are loaded
// before the first of the four calls, so the gathers overlap.  ReadOnly:
// the list was written by an earlier kernel (read through the read-only
// cache); false for records the calling thread has just written itself.
// Entries from `first` on (a multiple of 4).
template <bool ReadOnly = true, class F>
__device__ __forceinline__ void for_each_in_list(const int *base, int n, int i, int cnt,
                                                 const float4 *__restrict__ P, F &&f, int first = 0)
{
    const int4 *rec = reinterpret_cast<const int4 *>(base) + i;
    const size_t stride = (size_t)n;
    auto load = [&](int k) {
        const int4 *rp = rec + (size_t)(k >> 2) * stride;
        return ReadOnly ? __ldg(rp) : *rp;
    };
    int4 next = first < cnt ? load(first) : make_int4(0, 0, 0, 0);
#pragma unroll 1
    for (int k = first; k < cnt; k += 4) {
        const int4 r = next;
        if (k + 4 < cnt) next = load(k + 4);  // the next record loads while these four are summed
        const int m = min(4, cnt - k);
        const int j[4] = {r.x, r.y, r.z, r.w};
        float4 pj[4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (q < m) pj[q] = P[j[q]];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (q < m) f(j[q], pj[q]);
    }
}

// As for_each_in_list, with each entry's own data, fetch(j), loaded beside
// its position before the four calls: f(j, P[j], fetch(j)).
template <bool ReadOnly = true, class G, class F>
__device__ __forceinline__ void for_each_in_list_with(const int *base, int n, int i, int cnt,
                                                      const float4 *__restrict__ P, G &&fetch, F &&f, int first = 0)
{
    using T = decltype(fetch(0));
    const int4 *rec = reinterpret_cast<const int4 *>(base) + i;
    const size_t stride = (size_t)n;
    auto load = [&](int k) {
        const int4 *rp = rec + (size_t)(k >> 2) * stride;
        return ReadOnly ? __ldg(rp) : *rp;
    };
    int4 next = first < cnt ? load(first) : make_int4(0, 0, 0, 0);
#pragma unroll 1
    for (int k = first; k < cnt; k += 4) {
        const int4 r = next;
        if (k + 4 < cnt) next = load(k + 4);
        const int m = min(4, cnt - k);
        const int j[4] = {r.x, r.y, r.z, r.w};
        float4 pj[4];
        T xj[4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (q < m) {
                pj[q] = P[j[q]];
                xj[q] = fetch(j[q]);
            }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (q < m) f(j[q], pj[q], xj[q]);
    }
}

// Candidates [qb, e) of one (class, cell) run in class order, read from
// C.cls_pos.  test() sees a stand-in index that equals i only for particle i
// itself (tests compare it with i and nothing else); the body gets the sorted
// index, and skips sorted indices below jlo.  Slots: the body gets the class
// position q instead (no sorted index is looked up; jlo must be 0).
template <bool Split, bool Slots, class T, class B>
__device__ __forceinline__ void walk_run_cls(int qb, int e, int qi, int i, int jlo, const SimConsts &C, T &test,
                                             B &body)
{
    const float4 *__restrict__ src = C.cls_pos;
    const int *__restrict__ perm = C.cls_perm;
    if constexpr (!Split) {
#pragma unroll 1
        for (int q = qb; q < e; ++q) {
            const float4 pj = src[q];
            if (test(q == qi ? i : -1 - q, pj)) {
                if constexpr (Slots) {
                    body(q, pj);
                } else {
                    const int j = __ldg(perm + q);
                    if (j >= jlo) body(j, pj);
                }
            }
        }
    } else {
#pragma unroll 1
        for (int q0 = qb; q0 < e; q0 += 32) {
            const int cnt = min(32, e - q0);
            const float4 *s = src + q0;
            unsigned bits =
                chunk_bits(cnt, s, [&](int t, float4 p) { return test(q0 + t == qi ? i : -1 - (q0 + t), p); });
#pragma unroll 1
            while (bits) {
                const int t = __ffs(bits) - 1;
                bits &= bits - 1u;
                if constexpr (Slots) {
                    body(q0 + t, s[t]);
                } else {
                    const int j = __ldg(perm + q0 + t);
                    if (j >= jlo) body(j, s[t]);
                }
            }
        }
    }
}

// The 27-cell walk of real cell c over the alias classes (SimConsts::cls_perm):
// the same columns and pieces as the table walk, each piece restricted to the
// class of the real cells it covers.  A piece never spans two classes: z
// crosses a class boundary exactly where the table index wraps.  With lo > 0
// (candidates j >= lo only), a piece of i's own class starts at i's class
// position (class order keeps sorted order); other pieces filter in the body.
// Slots: the body gets class positions (walk_run_cls; lo must be 0).
// Ranged: only the cells of rg (the columns and z cells outside it skipped).
template <bool Split, bool Slots = false, bool Ranged = false, class T, class B>
__device__ __forceinline__ void walk_classes(int i, int3 c, int lo, const GridView &v, const SimConsts &C, T &test,
                                             B &body, CellRange rg = CellRange{})
{
    const unsigned m = v.mask;
    const unsigned D = (unsigned)v.D;
    const int sh = __ffs(v.D) - 1;
    const int qi = __ldg(C.cls_inv + i);
    const int ki = lo > 0 ? __ldg(C.cls_of + i) : -1;
    const int zl = Ranged ? c.z + rg.loz : c.z - 1, zh = Ranged ? c.z + rg.hiz : c.z + 1;
    const unsigned z0 = (unsigned)zl & m;
    const unsigned z2 = (unsigned)zh & m;
    // a range of 3 cells never starts and ends on one table cell (D >= 4)
    const bool wrap = (Ranged && zh - zl != 2) ? z0 > z2 : !(z0 < z2);
    const int kz0 = (zl >> sh) & 1, kz2 = (zh >> sh) & 1;
    const int *__restrict__ off = C.cls_off + v.base;
    const size_t keys = (size_t)C.cls_T;
#pragma unroll 1
    for (int col = 0; col < 9; ++col) {
        if constexpr (Ranged) {
            const int dx = col / 3 - 1, dy = col % 3 - 1;
            if (dx < rg.lox || dx > rg.hix || dy < rg.loy || dy > rg.hiy) continue;
        }
        const int xr = c.x + col / 3 - 1, yr = c.y + col % 3 - 1;
        const unsigned base = ((unsigned)xr & m) * D * D + ((unsigned)yr & m) * D;
        const int kxy = ((xr >> sh) & 1) | (((yr >> sh) & 1) << 1);
#pragma unroll 1
        for (int piece = 0; piece < (wrap ? 2 : 1); ++piece) {
            const unsigned za = (wrap && piece == 1) ? 0u : z0;
            const unsigned zb = wrap ? (piece == 0 ? D - 1 : z2) : z2;
            const int k = kxy | ((piece == 1 ? kz2 : kz0) << 2);
            const int *o = off + (size_t)k * keys + base;
            const int b = __ldg(o + za), e = __ldg(o + zb + 1);
            const bool own = k == ki;
            walk_run_cls<Split, Slots>(own ? max(b, qi) : b, e, qi, i, (lo > 0 && !own) ? lo : 0, C, test, body);
        }
    }
}

// Walk of particle i (sorted index) at position pi over the candidates
// j >= lo of its 27 cells on grid v: body(j, P[j]) for every j with
// test(j, P[j]).  S / g come from stage_block (S == nullptr or g < 0: no
// staging).  A particle whose Verlet list is valid (list_state) tests the
// list's entries instead, in their recorded (walk) order.  The pair arithmetic of the
// callers uses explicitly rounded operations, so every inlined copy of the
// pair functions produces the same bits.
// Ranged: only the cells of rg (the walk over its sub-range, or the Verlet
// list, whose entries are the full walk's).
template <bool Split, bool Ranged = false, class T, class B>
__device__ __forceinline__ void walk_neighbors(int i, float3 pi, int lo, const float4 *__restrict__ P,
                                               const GridView &v, const SimConsts &C, const StageShared *S, int g,
                                               T &&test, B &&body, CellRange rg = CellRange{})
{
    const int3 c = cell_of(pi, C);
    const unsigned m = v.mask;
    const unsigned D = (unsigned)v.D;
    const int *__restrict__ off = v.off;
    const bool staged = walks_staged(C, v, i, c, S, g);
    const int state = (C.vl && !C.vl_build) ? list_state(C, i, c, pi) : 1;
    if (C.nl_stats) atomicAdd(C.nl_stats + state, 1u);
    if (state == 0) {  // four entries at a time (measured faster than testing chunks first)
        for_each_in_list(C.vl, C.n, i, __ldg(C.vl_count + i), P, [&](int j, float4 pj) {
            if (j >= lo && test(j, pj)) body(j, pj);
        });
        return;
    }
    const unsigned z0 = (unsigned)(c.z + (Ranged ? rg.loz : -1)) & m;
    const unsigned z2 = (unsigned)(c.z + (Ranged ? rg.hiz : 1)) & m;

    if (C.cls_perm && !staged && __ldg(C.cls_moved) == 0) {
        if (C.nl_stats) atomicAdd(C.nl_stats + 4, 1u);
        walk_classes<Split, false, Ranged>(i, c, lo, v, C, test, body, rg);
        return;
    }

    // 27-cell walk: 9 column runs, split where z wraps around the table
    const bool wrap = (Ranged && rg.hiz - rg.loz != 2) ? z0 > z2 : !(z0 < z2);
#pragma unroll 1
    for (int col = 0; col < 9; ++col) {
        if constexpr (Ranged) {
            const int dx = col / 3 - 1, dy = col % 3 - 1;
            if (dx < rg.lox || dx > rg.hix || dy < rg.loy || dy > rg.hiy) continue;
        }
        const unsigned x = (unsigned)(c.x + col / 3 - 1) & m, y = (unsigned)(c.y + col % 3 - 1) & m;
        const unsigned base = x * D * D + y * D;
#pragma unroll 1
        for (int piece = 0; piece < (wrap ? 2 : 1); ++piece) {
            const unsigned za = (wrap && piece == 1) ? 0u : z0;
            const unsigned zb = wrap ? (piece == 0 ? D - 1 : z2) : z2;
            const int b = __ldg(off + base + za), e = __ldg(off + base + zb + 1);
            const int sidx = staged ? staged_index(*S, g, col, b, e) : -1;
            const float4 *src = sidx >= 0 ? S->pos + sidx : P + b;
            walk_run<Split>(max(b, lo), b, e, src, test, body);
        }
    }
}

// ---- recording walks over the walk planes (SimConsts::walk_xyz) ----

// Candidates [b, e) of one run, indices into the planes X, Y, Z: the q with
// |pi - p_q|^2 <= r2, in ascending q, as chunk(c0, bits) calls (q = c0 + t
// for each set bit t, chunks in ascending c0).  The run is read in quads
// aligned to 16 bytes, 32 candidates to a chunk mask (the candidates of a
// quad outside [b, e) are tested and dropped; the planes are padded by
// kPlanePad floats), and each paired fp32 operation serves two candidates.
// The squared distance has the bits len2(pi - pj) gives: pj + (-pi) is
// exactly -(pi - pj), its square the same, and each lane of a paired
// operation rounds as the scalar operation does.
template <class H>
__device__ __forceinline__ void record_run_planes(int b, int e, const float *__restrict__ X,
                                                  const float *__restrict__ Y, const float *__restrict__ Z,
                                                  float2 nx, float2 ny, float2 nz, float r2, H &chunk)
{
    if (b >= e) return;
#pragma unroll 1
    for (int c0 = b & ~3; c0 < e; c0 += 32) {
        const int cnt = min(32, e - c0);
        unsigned bits = 0u;
#pragma unroll 1
        for (int t = 0; t < cnt; t += 4 * kPlaneQuads) {
            float4 x[kPlaneQuads], y[kPlaneQuads], z[kPlaneQuads];
#pragma unroll
            for (int u = 0; u < kPlaneQuads; ++u) {
                x[u] = __ldg(reinterpret_cast<const float4 *>(X + c0 + t + 4 * u));
                y[u] = __ldg(reinterpret_cast<const float4 *>(Y + c0 + t + 4 * u));
                z[u] = __ldg(reinterpret_cast<const float4 *>(Z + c0 + t + 4 * u));
            }
            unsigned nib = 0u;
#pragma unroll
            for (int u = 0; u < kPlaneQuads; ++u) {
                const float2 xa = __fadd2_rn(make_float2(x[u].x, x[u].y), nx);
                const float2 xb = __fadd2_rn(make_float2(x[u].z, x[u].w), nx);
                const float2 ya = __fadd2_rn(make_float2(y[u].x, y[u].y), ny);
                const float2 yb = __fadd2_rn(make_float2(y[u].z, y[u].w), ny);
                const float2 za = __fadd2_rn(make_float2(z[u].x, z[u].y), nz);
                const float2 zb = __fadd2_rn(make_float2(z[u].z, z[u].w), nz);
                const float2 da = __ffma2_rn(za, za, __ffma2_rn(ya, ya, __fmul2_rn(xa, xa)));
                const float2 db = __ffma2_rn(zb, zb, __ffma2_rn(yb, yb, __fmul2_rn(xb, xb)));
                nib |= ((da.x <= r2 ? 1u : 0u) | (da.y <= r2 ? 2u : 0u) | (db.x <= r2 ? 4u : 0u) |
                        (db.y <= r2 ? 8u : 0u))
                       << (4 * u);
            }
            bits |= nib << t;
        }
        bits &= ~0u << max(b - c0, 0);        // below the run (first chunk only)
        if (cnt < 32) bits &= (1u << cnt) - 1u;  // past its end
        if (bits) chunk(c0, bits);
    }
}

// The recording walk of a particle at pi over the walk planes, unstaged and
// without Verlet lists, for the test |pi - pj|^2 <= r2: the hits in walk
// order, as chunk(c0, bits) calls (record_run_planes).
// order 2 (classes on): the pieces of walk_classes, q a class position;
// order 1: the table walk of walk_neighbors, q a sorted index.  Counted in
// C.nl_stats as those walks count.
template <class H>
__device__ __forceinline__ void record_walk_planes(int order, float3 pi, float r2, const GridView &v,
                                                   const SimConsts &C, H &&chunk)
{
    const size_t st = (size_t)C.walk_stride;
    const float *__restrict__ X = C.walk_xyz;
    const float *__restrict__ Y = X + st;
    const float *__restrict__ Z = Y + st;
    const float2 nx = make_float2(-pi.x, -pi.x), ny = make_float2(-pi.y, -pi.y), nz = make_float2(-pi.z, -pi.z);
    if (C.nl_stats) {
        atomicAdd(C.nl_stats + 1, 1u);
        if (order == 2) atomicAdd(C.nl_stats + 4, 1u);
    }
    const int3 c = cell_of(pi, C);
    const unsigned m = v.mask;
    const unsigned D = (unsigned)v.D;
    const unsigned z0 = (unsigned)(c.z - 1) & m;
    const unsigned z2 = (unsigned)(c.z + 1) & m;
    const bool wrap = !(z0 < z2);
    if (order == 2) {
        const int sh = __ffs(v.D) - 1;
        const int kz0 = ((c.z - 1) >> sh) & 1, kz2 = ((c.z + 1) >> sh) & 1;
        const int *__restrict__ off = C.cls_off + v.base;
        const size_t keys = (size_t)C.cls_T;
#pragma unroll 1
        for (int col = 0; col < 9; ++col) {
            const int xr = c.x + col / 3 - 1, yr = c.y + col % 3 - 1;
            const unsigned base = ((unsigned)xr & m) * D * D + ((unsigned)yr & m) * D;
            const int kxy = ((xr >> sh) & 1) | (((yr >> sh) & 1) << 1);
#pragma unroll 1
            for (int piece = 0; piece < (wrap ? 2 : 1); ++piece) {
                const unsigned za = (wrap && piece == 1) ? 0u : z0;
                const unsigned zb = wrap ? (piece == 0 ? D - 1 : z2) : z2;
                const int k = kxy | ((piece == 1 ? kz2 : kz0) << 2);
                const int *o = off + (size_t)k * keys + base;
                record_run_planes(__ldg(o + za), __ldg(o + zb + 1), X, Y, Z, nx, ny, nz, r2, chunk);
            }
        }
    } else {
        const int *__restrict__ off = v.off;
#pragma unroll 1
        for (int col = 0; col < 9; ++col) {
            const unsigned x = (unsigned)(c.x + col / 3 - 1) & m, y = (unsigned)(c.y + col % 3 - 1) & m;
            const unsigned base = x * D * D + y * D;
#pragma unroll 1
            for (int piece = 0; piece < (wrap ? 2 : 1); ++piece) {
                const unsigned za = (wrap && piece == 1) ? 0u : z0;
                const unsigned zb = wrap ? (piece == 0 ? D - 1 : z2) : z2;
                record_run_planes(__ldg(off + base + za), __ldg(off + base + zb + 1), X, Y, Z, nx, ny, nz, r2, chunk);
            }
        }
    }
}

}  // namespace bp
