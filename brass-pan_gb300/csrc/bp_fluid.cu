// bp_fluid.cu -- position-based fluid passes (gather form, fixed neighbour order).
//
// Reference kernels (brasstower/kernel/fluid.cuh):
//   fluidLambda (:78-159)              -> k_lambda
//   fluidPosition (:161-228) + accDevArr_float3 (kernel/util.cuh:261-269)
//                                      -> k_deltap (gather, no atomics, epilogue fused)
//   fluidOmega (:231-279) + fluidNormal (:387-434)            -> k_post_a (one walk)
//   fluidVorticity (:281-336) + fluidAkinciTension (:436-488) -> k_post_b (one walk)
//   fluidXSph (:338-385)                                      -> k_post_c
//
// The reference scatters each pair's position correction to both particles
// with float atomics; here every particle gathers its own sum over the same
// pairs in a fixed order, so results are deterministic run to run.  The pair
// term for (k, j) is bit-identical to the reference's term for (j, k) up to
// sign, because the spiky gradient is odd in the difference vector.
#include "bp_internal.h"
#include "bp_walk.cuh"

namespace bp {

constexpr int kScanThreads = kWalkThreads;  // scan kernels stage their neighbourhood (bp_walk.cuh)

// CTAs per SM the list-reading passes are compiled for.  The position pass
// loads each record's four positions and (lambda, mass) pairs before its four
// pair terms; at 4 CTAs (64 registers) that measured faster than at 5 (48
// registers, spilling), and than 5 CTAs with the pairs loaded per term
// (mixed scene 9.86 -> 9.68 ms per frame early, 15.40 -> 15.17 late).
#ifndef BP_DELTAP_MIN_BLOCKS
#define BP_DELTAP_MIN_BLOCKS 4
#endif
// Passes B and C load each record's neighbour data (|omega| and normal, or
// velocity) with the positions before the four pair terms; at 3 CTAs (80
// registers) that measured faster than at 4 (64, spilling) and than 4 CTAs
// with the data loaded per term (mixed scene 9.75 -> 9.62 ms per frame early,
// 15.24 -> 15.09 late).
#ifndef BP_POSTBC_MIN_BLOCKS
#define BP_POSTBC_MIN_BLOCKS 3
#endif

// Ends the Verlet list build of particle i (SimConsts::vl): its count, and
// the cell and position the list holds for (cell -1: no list, because it
// overflowed or the particle's column runs wrap around the table).
__device__ __forceinline__ void finish_verlet(const SimConsts &C, int i, float4 pi4, int cnt)
{
    const int3 c = cell_of(f3(pi4), C);
    const unsigned z0 = (unsigned)(c.z - 1) & C.mask, z2 = (unsigned)(c.z + 1) & C.mask;
    C.vl_count[i] = cnt;
    C.nl_pos[i] = pi4;
    C.nl_cell[i] = (cnt >= 0 && z0 < z2) ? cell_addr(c.x, c.y, c.z, C.D, C.mask) : -1;
}

// Reference mode (Q1): density sums only sorted indices j >= i; solid
// neighbours count x solid_scale; C = rho/rho0 - 1, clamped at 0 when Akinci
// is on; lambda = -C / lambda_den.  Textbook mode: all j, exact denominator.
//
// With C.nbr (neighbour lists on) the walk also records, for the position
// pass that reads the same positions, every j with r^2 <= h^2 in walk order
// (all j, also below i; solids too in reference mode, whose position pass
// gathers from fluid neighbours).  With C.vl_build it records the substep's
// Verlet lists instead: every j within h + skin.
template <bool Split, bool Stage>
__device__ __forceinline__ void k_lambda_tile(
    const SimConsts &C,
    const float4 *__restrict__ P,
    const float *__restrict__ mass,
    const int *__restrict__ off,
    float *__restrict__ lam,
    float *__restrict__ rho,
    int i0)
{
    StageShared &S = stage_shared();
    const int g = Stage ? stage_block(C, P, off, i0, S) : -1;
    const int t = i0 + threadIdx.x;  // the slot of the position pass's list
    if (t >= C.n) return;
    const int i = Stage ? t : walker_index(C, t);
    const float4 pi4 = P[i];
    const bool build = C.vl_build != 0;
    const bool rec = build || C.nbr != nullptr;
    // Slot lists: while the threads take class order (and no Verlet list can
    // stand in for a walk) the list holds class positions, and the position
    // pass gathers positions, masses and lambdas from the class-order copies.
    const bool slots = !Stage && C.nbr && !build && !C.vl && classes_on(C);
    const bool solid = phase_of(pi4) > 0;
    // (lambda, mass) for the position pass's gathers: by slot with slot
    // lists, by sorted index with lists of sorted indices
    auto put_lm = [&](float l) {
        if (slots) C.cls_lm[t] = make_float2(l, __ldg(mass + i));
        else if (C.lm && !build) C.lm[i] = make_float2(l, __ldg(mass + i));
    };
    if (solid) {  // solids carry lambda 0 (read by the position pass)
        lam[i] = 0.f;
        put_lm(0.f);
    }
    if (solid && (C.textbook || !rec)) {
        if (build) C.nl_cell[i] = -1;
        return;
    }
    const int sc = scene_index(C, i);
    const GridView v = grid_view(C, sc, off);
    const float rho0 = rest_density(C, sc);
    const float3 pi = f3(pi4);
    const float r2 = build ? C.nl_hs2 : C.h2;
    float density = 0.f;
    // Verlet lists are kept per particle, the position pass's lists per slot
    ListWriter list(build ? C.vl : C.nbr, build ? C.vl_cap : C.nbr_cap, C.n, build ? i : t);
    auto finish = [&]() {
        const int cnt = list.finish();
        if (build) finish_verlet(C, i, pi4, cnt);
        else C.nbr_count[t] = cnt;
    };
    auto record = [&](int &self) {  // entries: sorted indices, or class positions (slots)
        auto push = [&](int j, float4) {
            if (j == (slots ? t : i)) self = list.cnt;
            list.push(j);
        };
        auto test = [&](int, float4 pj) { return len2(pi - f3(pj)) <= r2; };
        // the walk planes hold the order this walk reads (class positions with
        // slots, sorted indices otherwise): the same hits in the same order
        const int planes = (Split && !Stage && !C.vl) ? walk_planes_order(C) : 0;
        if (planes == (slots ? 2 : 1)) {
            const int me = slots ? t : i;  // the particle's own entry
            record_walk_planes(planes, pi, r2, v, C, [&](int c0, unsigned bits) {
                const unsigned d = (unsigned)(me - c0);
                if (d < 32u && ((bits >> d) & 1u)) self = list.cnt + __popc(bits & ((1u << d) - 1u));
                list.push_bits(c0, bits);
            });
        } else if (slots) {  // the class walk walk_neighbors would take (no staging, no Verlet list), counted alike
            if (C.nl_stats) {
                atomicAdd(C.nl_stats + 1, 1u);
                atomicAdd(C.nl_stats + 4, 1u);
            }
            walk_classes<Split, true>(i, cell_of(pi, C), 0, v, C, test, push);
        } else {
            walk_neighbors<Split>(i, pi, 0, P, v, C, Stage ? &S : nullptr, g, test, push);
        }
        const int cnt = list.finish();
        C.nbr_count[t] = cnt;
        return cnt;
    };
    if (!C.textbook) {
        auto dens_m = [&](float mj, float4 pj) {
            const float ld = __fmul_rn(mj, poly6(C, len2(pi - f3(pj))));
            density = __fadd_rn(density, (phase_of(pj) < 0) ? ld : __fmul_rn(C.solid_scale, ld));
        };
        auto dens = [&](int j, float4 pj) { dens_m(__ldg(mass + j), pj); };
        auto test = [&](int, float4 pj) { return len2(pi - f3(pj)) <= r2; };
        if (C.nbr && !build) {
            // record first, then sum the density over the list's j >= i (the
            // mass gathers overlap there); an overflowed list walks again.
            // Where no column run wraps around the table the walk visits j in
            // ascending order, so the j >= i are the entries from i itself on.
            int self = 0;
            const int cnt = record(self);
            if (solid) return;
            const int3 c = cell_of(pi, C);
            auto inner = [&](int a) {
                const unsigned u = (unsigned)a & v.mask;
                return u != 0u && u != v.mask;
            };
            const bool ascending = inner(c.x) && inner(c.y) && inner(c.z);
            const int first = ascending ? (self & ~3) : 0;
            if (cnt >= 0 && slots) {
                int e = first;  // entry index: ascending, the j >= i are the entries from self on
                for_each_in_list<false>(C.nbr, C.n, t, cnt, C.cls_pos, [&](int q, float4 pj) {
                    const bool upper = ascending ? e >= self : __ldg(C.cls_perm + q) >= i;
                    ++e;
                    if (upper) dens_m(__ldg(C.cls_mass + q), pj);
                }, first);
            } else if (cnt >= 0) {
                for_each_in_list<false>(C.nbr, C.n, t, cnt, P, [&](int j, float4 pj) {
                    if (j >= i) dens(j, pj);
                }, first);
            } else {
                walk_neighbors<Split>(i, pi, i, P, v, C, Stage ? &S : nullptr, g, test, dens);
            }
        } else {
            walk_neighbors<Split>(i, pi, rec ? 0 : i, P, v, C, Stage ? &S : nullptr, g, test,
                                  [&](int j, float4 pj) {
                                      if (rec) list.push(j);
                                      if (solid || j < i || (build && !(len2(pi - f3(pj)) <= C.h2))) return;
                                      dens(j, pj);
                                  });
            if (rec) finish();
        }
        if (solid) return;
        float c = density / rho0 - 1.0f;
        if (C.clamp_c) c = fmaxf(c, 0.0f);
        lam[i] = -c / C.lambda_den;
        put_lm(lam[i]);
    } else {
        const float inv_rho0 = inv_rest_density(C, sc);
        float sum_g2 = 0.f;
        float3 gi = make_float3(0.f, 0.f, 0.f);
        const float *mw = slots ? C.cls_mass : mass;  // indexed by the list's entries
        auto term = [&](int j, float4 pj) {
            const float3 diff = pi - f3(pj);
            const float d2 = len2(diff);
            const float mj = __ldg(mw + j);
            const float ld = __fmul_rn(mj, poly6(C, d2));
            density = __fadd_rn(density, (phase_of(pj) < 0) ? ld : __fmul_rn(C.solid_scale, ld));
            if (d2 > 0.f) {
                const float3 g = __fmul_rn(-mj, inv_rho0) * spiky_grad_r(C, diff, d2, rsqrtf(d2));
                sum_g2 = __fadd_rn(sum_g2, dot3(g, g));
                gi -= g;
            }
        };
        auto test = [&](int, float4 pj) { return len2(pi - f3(pj)) <= r2; };
        if (C.nbr && !build) {  // record first, then sum over the list (as above)
            int self = 0;
            const int cnt = record(self);
            if (cnt >= 0) {
                for_each_in_list<false>(C.nbr, C.n, t, cnt, slots ? C.cls_pos : P, term);
            } else {
                mw = mass;  // the walk gives sorted indices
                walk_neighbors<Split>(i, pi, 0, P, v, C, Stage ? &S : nullptr, g, test, term);
            }
        } else {
            walk_neighbors<Split>(i, pi, 0, P, v, C, Stage ? &S : nullptr, g, test, [&](int j, float4 pj) {
                if (rec) list.push(j);
                if (build && !(len2(pi - f3(pj)) <= C.h2)) return;
                term(j, pj);
            });
            if (rec) finish();
        }
        float c = density / rho0 - 1.0f;
        if (C.clamp_c) c = fmaxf(c, 0.0f);
        sum_g2 += dot3(gi, gi);
        lam[i] = -c / (sum_g2 + C.relaxation);
        put_lm(lam[i]);
    }
    rho[i] = density;
    if (slots) C.cls_rho[t] = density;
}

template <bool Split, bool Stage, bool Persist = false>
__global__ void __launch_bounds__(kScanThreads, BP_SCAN_MIN_BLOCKS) k_lambda(
    SimConsts C,
    const float4 *__restrict__ P,
    const float *__restrict__ mass,
    const int *__restrict__ off,
    float *__restrict__ lam,
    float *__restrict__ rho)
{
    // one tile of blockDim.x particles per CTA, or, persistent (an unstaged
    // launch of at most one resident wave: SimConsts::scan_persist), every
    // gridDim.x-th tile from blockIdx.x on
    if constexpr (Persist) {
        for (int i0 = blockIdx.x * blockDim.x; i0 < C.n; i0 += gridDim.x * blockDim.x)
            k_lambda_tile<Split, Stage>(C, P, mass, off, lam, rho, i0);
    } else {
        k_lambda_tile<Split, Stage>(C, P, mass, off, lam, rho, blockIdx.x * blockDim.x);
    }
}

// Kernels with a split walk (test, then body over the hits) and a fused one.
// Kernels instantiated for split / fused walks and staged / unstaged CTAs
// (an unstaged instantiation carries none of the staging code or registers).
// Persistent launches (SimConsts::scan_persist) exist for the split,
// unstaged instantiation, the one the autotuner keeps almost everywhere.
#define BP_LAUNCH_SPLIT(kernel, st, ...)                                                              \
    do {                                                                                              \
        const size_t smem_ = stage_bytes(C);                                                          \
        if (C.split && C.stage) launch_scan(kernel<true, true>, C, smem_, st, __VA_ARGS__);           \
        else if (C.split && C.scan_persist) launch_scan(kernel<true, false, true>, C, smem_, st, __VA_ARGS__); \
        else if (C.split) launch_scan(kernel<true, false>, C, smem_, st, __VA_ARGS__);                \
        else if (C.stage) launch_scan(kernel<false, true>, C, smem_, st, __VA_ARGS__);                \
        else launch_scan(kernel<false, false>, C, smem_, st, __VA_ARGS__);                            \
    } while (0)

void launch_lambda(cudaStream_t st, const SimConsts &C, const float4 *P, const float *mass, const int *off,
                   float *lam, float *rho, LaunchLog *L)
{
    if (C.n <= 0) return;
    BP_LAUNCH_SPLIT(k_lambda, st, C, P, mass, off, lam, rho);
    L->done(__func__);
}

// Position correction.  Reference mode: the pair (a, b), a < b, contributes
// when a is a fluid particle (only fluid threads run fluidPosition and they
// only visit b > a), to both ends.  In gather form particle k includes j when
// the lower-indexed of (k, j) is fluid.  Textbook mode: fluid k gathers over
// every neighbour; solids do not move.  With C.nbr the neighbours come from
// the lists k_lambda recorded at the same positions (r^2 <= h^2, walk order);
// particles whose list overflowed walk their cells.
template <bool Split, bool Stage>
__device__ __forceinline__ void k_deltap_tile(
    const SimConsts &C,
    DeltaArgs a,
    int i0)
{
    StageShared &S = stage_shared();
    const int t = i0 + threadIdx.x;  // the slot of k's list (k_lambda)
    const bool valid = t < C.n;
    const int k = (Stage || !valid) ? t : walker_index(C, t);
    const float4 pk4 = valid ? a.P[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int phk = phase_of(pk4);
    const bool moves = valid && !(C.textbook && phk > 0);
    const int listed = (moves && C.nbr) ? __ldg(C.nbr_count + t) : -1;
    const bool walk = moves && listed < 0;
    const int g = (Stage && __syncthreads_or(walk)) ? stage_block(C, a.P, a.off, i0, S) : -1;
    if (!valid) return;
    const float3 pk = f3(pk4);
    const int sc = scene_index(C, k);
    float3 sum = make_float3(0.f, 0.f, 0.f);
    if (moves) {
        const float lk = a.lam[k];
        auto pair = [&](float4 pj4, float lj, float mj) {
            const float3 diff = pk - f3(pj4);
            const float d2 = len2(diff);
            float sl = __fadd_rn(lk, lj);
            if (C.scorr_on)
                sl = __fsub_rn(sl, __fmul_rn(C.scorr_k, ipowf(__fmul_rn(poly6(C, d2), C.scorr_inv_wq), C.scorr_ni)));
            float3 delta = sl * spiky_grad_r(C, diff, d2, rsqrtf(d2));
            if (C.delta_clamp > 0.f) {  // per-pair clamp; the length is only needed past it
                const float l2 = len2(delta);
                if (!(l2 < C.delta_clamp2)) delta = delta * __fmul_rn(C.delta_clamp, rsqrtf(l2));
            }
            sum = fma3(mj, delta, sum);
        };
        auto body = [&](int j, float4 pj4) {
            if (!C.textbook && !((j > k) ? (phk < 0) : (phase_of(pj4) < 0))) return;
            pair(pj4, __ldg(a.lam + j), __ldg(a.mass + j));
        };
        // slot lists (k_lambda) hold class positions q: the pair's data come
        // from the class-order copies, the sorted index only where one of the
        // two is a solid (the fluid-fluid pairs pass the rule either way)
        const bool slots = !Stage && C.nbr && !C.vl && classes_on(C);
        // each entry's (lambda, mass) loads with its position, before the
        // four pair terms of a record
        if (!walk && slots) {
            auto fetch = [&](int q) { return __ldg(C.cls_lm + q); };
            for_each_in_list_with(C.nbr, C.n, t, listed, C.cls_pos, fetch, [&](int q, float4 pj4, float2 lm) {
                if (!(len2(pk - f3(pj4)) > 0.f)) return;  // r = 0 excludes k itself
                if (!C.textbook) {
                    const bool fj = phase_of(pj4) < 0;
                    if (!(phk < 0 && fj)) {
                        const int j = __ldg(C.cls_perm + q);
                        if (!((j > k) ? (phk < 0) : fj)) return;
                    }
                }
                pair(pj4, lm.x, lm.y);
            });
        } else if (!walk && C.lm) {
            auto fetch = [&](int j) { return __ldg(C.lm + j); };
            for_each_in_list_with(C.nbr, C.n, t, listed, a.P, fetch, [&](int j, float4 pj4, float2 lm) {
                if (!(len2(pk - f3(pj4)) > 0.f)) return;  // r = 0 excludes k itself
                if (!C.textbook && !((j > k) ? (phk < 0) : (phase_of(pj4) < 0))) return;
                pair(pj4, lm.x, lm.y);
            });
        } else if (!walk) {
            auto listed_body = [&](int j, float4 pj4) {  // r = 0 excludes k itself
                if (len2(pk - f3(pj4)) > 0.f) body(j, pj4);
            };
            for_each_in_list(C.nbr, C.n, t, listed, a.P, listed_body);
        } else {
            walk_neighbors<Split>(
                k, pk, 0, a.P, grid_view(C, sc, a.off), C, Stage ? &S : nullptr, g,
                [&](int, float4 pj4) {  // r = 0 excludes k itself
                    const float d2 = len2(pk - f3(pj4));
                    return d2 <= C.h2 && d2 > 0.f;
                },
                body);
        }
    }
    float3 p = pk + sum * inv_rest_density(C, sc);
    if (a.epilogue == 1) {
        plane_collide(C, sc, f3(a.Xs[k]), p);
    } else if (a.epilogue == 2) {  // updateVelocity + updatePositions (PS:71-81, 121-137)
        const float4 xs = a.Xs[k];
        const float3 v = (p - f3(xs)) * C.inv_dt;
        a.Xc[k] = make_float4(p.x, p.y, p.z, xs.w);
        a.Vc[k] = make_float4(v.x, v.y, v.z, pk4.w);
        a.orig_c[k] = a.orig_s[k];
    }
    a.Pout[k] = make_float4(p.x, p.y, p.z, pk4.w);
    track_displacement(C, k, p, true);
}

template <bool Split, bool Stage, bool Persist = false>
__global__ void __launch_bounds__(kScanThreads, BP_DELTAP_MIN_BLOCKS) k_deltap(
    SimConsts C,
    DeltaArgs a)
{
    // one tile of blockDim.x particles per CTA, or, persistent (an unstaged
    // launch of at most one resident wave: SimConsts::scan_persist), every
    // gridDim.x-th tile from blockIdx.x on
    if constexpr (Persist) {
        for (int i0 = blockIdx.x * blockDim.x; i0 < C.n; i0 += gridDim.x * blockDim.x)
            k_deltap_tile<Split, Stage>(C, a, i0);
    } else {
        k_deltap_tile<Split, Stage>(C, a, blockIdx.x * blockDim.x);
    }
}

void launch_deltap(cudaStream_t st, const SimConsts &C, const DeltaArgs &a, LaunchLog *L)
{
    if (C.n <= 0) return;
    BP_LAUNCH_SPLIT(k_deltap, st, C, a);
    L->done(__func__);
}

// The post passes keep class positions in their lists (SimConsts::cls_post):
// pass A records them and every pass reads its neighbours' data from the
// class-order copies, as k_lambda and k_deltap do.
__device__ __forceinline__ bool post_slots(const SimConsts &C, bool stage)
{
    return !stage && C.cls_post && C.nbr && C.nbr_count && !C.vl && classes_on(C);
}

// Pass A: vorticity omega_i (fluidOmega) and Akinci normal n_i (fluidNormal)
// in one walk over same-phase neighbours with 0 < r^2 <= h^2.
// Om[i] = (omega, |omega|); Nm[i] = (h * n, rho_i).
template <bool Split, bool Stage>
__device__ __forceinline__ void k_post_a_tile(
    const SimConsts &C,
    const float4 *__restrict__ P,
    const float4 *__restrict__ V,
    const float *__restrict__ rho,
    const int *__restrict__ off,
    float4 *__restrict__ Om,
    float4 *__restrict__ Nm,
    int i0)
{
    StageShared &S = stage_shared();
    const int g = Stage ? stage_block(C, P, off, i0, S) : -1;
    const int t = i0 + threadIdx.x;  // the slot of the list passes B and C read
    if (t >= C.n) return;
    const int i = Stage ? t : walker_index(C, t);
    const float4 pi4 = P[i];
    const int phi = phase_of(pi4);
    if (phi >= 0) return;
    const float3 pi = f3(pi4);
    const float3 vi = f3(V[i]);
    float3 om = make_float3(0.f, 0.f, 0.f), nn = make_float3(0.f, 0.f, 0.f);
    const bool want_om = C.use_vort, want_n = C.use_akinci;
    const bool slots = post_slots(C, Stage);
    auto term_at = [&](const float4 *__restrict__ Vp, const float *__restrict__ rp, int j, float4 pj4) {
        const float3 diff = pi - f3(pj4);
        const float d2 = len2(diff);
        if (!(d2 > 0.f)) return;
        const float3 g = spiky_grad_r(C, diff, d2, rsqrtf(d2));
        if (want_om) om += cross3(f3(Vp[j]) - vi, g);
        if (want_n) nn = fma3(__frcp_rn(__ldg(rp + j)), g, nn);
    };
    auto term = [&](int j, float4 pj4) { term_at(V, rho, j, pj4); };
    const GridView v = grid_view(C, scene_index(C, i), off);
    auto test = [&](int, float4 pj4) { return len2(pi - f3(pj4)) <= C.h2; };
    // The walk takes the passes' common neighbours (r = 0 included, as pass C
    // wants them).  With lists on it only records them (for passes B and C as
    // well), and the terms are then summed over the list four neighbours at a
    // time, so their velocity and density gathers overlap; a list that
    // overflowed is summed by walking again.
    int cnt = -1;
    if (C.nbr) {
        ListWriter list(C.nbr, C.nbr_cap, C.n, t);
        // the walk planes hold the order this walk reads (class positions with
        // slots, sorted indices otherwise): the same hits in the same order,
        // each chunk's kept where the phase plane matches and not the own entry
        const int planes = (Split && !Stage && !C.vl) ? walk_planes_order(C) : 0;
        if (planes == (slots ? 2 : 1)) {
            const int *__restrict__ W = reinterpret_cast<const int *>(C.walk_xyz) + 3 * (size_t)C.walk_stride;
            const int me = slots ? t : i;
            record_walk_planes(planes, pi, C.h2, v, C, [&](int c0, unsigned bits) {
                const unsigned d = (unsigned)(me - c0);
                if (d < 32u) bits &= ~(1u << d);
                unsigned same = 0u;
                for (unsigned quads = bits; quads;) {  // the phases of the quads holding hits
                    const int q4 = (__ffs(quads) - 1) & ~3;
                    const int4 w = __ldg(reinterpret_cast<const int4 *>(W + c0 + q4));
                    same |= ((w.x == phi ? 1u : 0u) | (w.y == phi ? 2u : 0u) | (w.z == phi ? 4u : 0u) |
                             (w.w == phi ? 8u : 0u))
                            << q4;
                    quads &= ~(0xfu << q4);
                }
                list.push_bits(c0, bits & same);
            });
        } else if (slots) {  // the class walk walk_neighbors would take, recording class positions
            if (C.nl_stats) {
                atomicAdd(C.nl_stats + 1, 1u);
                atomicAdd(C.nl_stats + 4, 1u);
            }
            auto push = [&](int q, float4 pj4) {
                if (q != t && phase_of(pj4) == phi) list.push(q);
            };
            walk_classes<Split, true>(i, cell_of(pi, C), 0, v, C, test, push);
        } else {
            walk_neighbors<Split>(i, pi, 0, P, v, C, Stage ? &S : nullptr, g, test, [&](int j, float4 pj4) {
                if (j != i && phase_of(pj4) == phi) list.push(j);
            });
        }
        cnt = list.finish();
        C.nbr_count[t] = cnt;
        // the records just written come back through the coherent path (plain loads)
        if (cnt >= 0 && slots)
            for_each_in_list<false>(C.nbr, C.n, t, cnt, C.cls_pos,
                                    [&](int q, float4 pj4) { term_at(C.cls_vel, C.cls_rho, q, pj4); });
        else if (cnt >= 0)
            for_each_in_list<false>(C.nbr, C.n, t, cnt, P, term);
    }
    if (cnt < 0)
        walk_neighbors<Split>(i, pi, 0, P, v, C, Stage ? &S : nullptr, g, test, [&](int j, float4 pj4) {
            if (j != i && phase_of(pj4) == phi) term(j, pj4);
        });
    const float4 om4 = make_float4(om.x, om.y, om.z, len3(om));
    const float3 n = C.h * nn;
    const float4 nm4 = make_float4(n.x, n.y, n.z, rho[i]);
    Om[i] = om4;
    Nm[i] = nm4;
    if (slots) {
        C.cls_om[t] = om4;
        C.cls_nm[t] = nm4;
    }
}

template <bool Split, bool Stage, bool Persist = false>
__global__ void __launch_bounds__(kScanThreads, BP_SCAN_MIN_BLOCKS) k_post_a(
    SimConsts C,
    const float4 *__restrict__ P,
    const float4 *__restrict__ V,
    const float *__restrict__ rho,
    const int *__restrict__ off,
    float4 *__restrict__ Om,
    float4 *__restrict__ Nm)
{
    // one tile of blockDim.x particles per CTA, or, persistent (an unstaged
    // launch of at most one resident wave: SimConsts::scan_persist), every
    // gridDim.x-th tile from blockIdx.x on
    if constexpr (Persist) {
        for (int i0 = blockIdx.x * blockDim.x; i0 < C.n; i0 += gridDim.x * blockDim.x)
            k_post_a_tile<Split, Stage>(C, P, V, rho, off, Om, Nm, i0);
    } else {
        k_post_a_tile<Split, Stage>(C, P, V, rho, off, Om, Nm, blockIdx.x * blockDim.x);
    }
}

// Passes B and C: the number of recorded neighbours of particle i (its list
// in slot t, k_post_a), or kWalkCells when it must walk its cells (no lists,
// or they overflowed).  Solids and indices past the end need neither (0).
constexpr int kWalkCells = -1;
__device__ __forceinline__ int post_list_count(const SimConsts &C, const float4 *__restrict__ P, int i, int t)
{
    if (i >= C.n || phase_of(P[i]) >= 0) return 0;
    if (!C.nbr || !C.nbr_count) return kWalkCells;
    const int cnt = __ldg(C.nbr_count + t);
    return cnt >= 0 ? cnt : kWalkCells;
}

// Pass B: vorticity confinement (fluidVorticity) then Akinci tension
// (fluidAkinciTension), both on the same neighbours.  v' = v + eps (N x w) dt,
// v'' = v' + F dt, exactly the reference's sequence (in-place update followed
// by newVelocities = velocities + F dt).  Solids pass through.
template <bool Split, bool Stage>
__device__ __forceinline__ void k_post_b_tile(
    const SimConsts &C,
    const float4 *__restrict__ P,
    const float4 *__restrict__ V,
    const float4 *__restrict__ Om,
    const float4 *__restrict__ Nm,
    const int *__restrict__ off,
    float4 *__restrict__ Vout,
    int i0)
{
    StageShared &S = stage_shared();
    const int t = i0 + threadIdx.x;
    const int i = (Stage || t >= C.n) ? t : walker_index(C, t);
    const int cnt = post_list_count(C, P, i, t);
    const int g = (Stage && __syncthreads_or(cnt == kWalkCells)) ? stage_block(C, P, off, i0, S) : -1;
    if (i >= C.n) return;
    const float4 pi4 = P[i];
    const float4 vi4 = V[i];
    const int phi = phase_of(pi4);
    if (phi >= 0) {
        Vout[i] = vi4;
        return;
    }
    const int sc = scene_index(C, i);
    const float two_rho0 = 2.0f * rest_density(C, sc);
    const float3 pi = f3(pi4);
    const float4 ni4 = Nm[i];
    const float3 ni = f3(ni4);
    const float rhoi = ni4.w;
    float3 eta = make_float3(0.f, 0.f, 0.f), ft = make_float3(0.f, 0.f, 0.f);
    const bool want_v = C.use_vort, want_t = C.use_akinci;
    const bool slots = post_slots(C, Stage);
    // a neighbour's |omega| and (h n, rho), as the pair terms read them
    struct Nb {
        float om;
        float4 nm;
    };
    auto fetch_at = [&](const float4 *__restrict__ Omp, const float4 *__restrict__ Nmp, int j) {
        Nb r;
        r.om = want_v ? Omp[j].w : 0.f;
        r.nm = want_t ? Nmp[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        return r;
    };
    auto pair_terms = [&](float4 pj4, const Nb &nb) {
        const float3 diff = pi - f3(pj4);
        const float d2 = len2(diff);
        if (!(d2 > 0.f)) return;
        const float inv_r = rsqrtf(d2);
        if (want_v) eta = fma3(nb.om, spiky_grad_r(C, diff, d2, inv_r), eta);
        if (want_t) {
            const float4 nj4 = nb.nm;
            const float dist = __fmul_rn(d2, inv_r);
            const float3 fco = __fmul_rn(__fmul_rn(-C.tension, akinci_spline(C, dist)), inv_r) * diff;
            const float3 fcu = (-C.tension) * (ni - f3(nj4));
            const float kij = __fmul_rn(two_rho0, __frcp_rn(__fadd_rn(rhoi, nj4.w)));
            ft = fma3(kij, fco + fcu, ft);
        }
    };
    auto body = [&](int j, float4 pj4) { pair_terms(pj4, fetch_at(Om, Nm, j)); };
    // each entry's omega and normal load with its position, before the four
    // pair terms of a record
    auto listed = [&](int, float4 pj4, const Nb &nb) { pair_terms(pj4, nb); };
    if (cnt != kWalkCells && slots) {
        for_each_in_list_with(C.nbr, C.n, t, cnt, C.cls_pos,
                              [&](int q) { return fetch_at(C.cls_om, C.cls_nm, q); }, listed);
    } else if (cnt != kWalkCells) {
        for_each_in_list_with(C.nbr, C.n, t, cnt, P, [&](int j) { return fetch_at(Om, Nm, j); }, listed);
    } else {
        walk_neighbors<Split>(
            i, pi, 0, P, grid_view(C, sc, off), C, Stage ? &S : nullptr, g,
            [&](int j, float4 pj4) { return j != i && phase_of(pj4) == phi && len2(pi - f3(pj4)) <= C.h2; },
            body);
    }
    float3 v = f3(vi4);
    if (want_v && len2(eta) > 1e-3f) {
        const float inv = 1.0f / sqrtf(dot3(eta, eta));
        const float3 nrm = eta * inv;
        v += (C.vort_eps * cross3(nrm, f3(Om[i]))) * C.dt;
    }
    if (want_t) v = v + ft * C.dt;
    const float4 v4 = make_float4(v.x, v.y, v.z, vi4.w);
    Vout[i] = v4;
    if (slots) C.cls_vb[t] = v4;  // pass C's neighbour velocities
}

template <bool Split, bool Stage, bool Persist = false>
__global__ void __launch_bounds__(kScanThreads, BP_POSTBC_MIN_BLOCKS) k_post_b(
    SimConsts C,
    const float4 *__restrict__ P,
    const float4 *__restrict__ V,
    const float4 *__restrict__ Om,
    const float4 *__restrict__ Nm,
    const int *__restrict__ off,
    float4 *__restrict__ Vout)
{
    // one tile of blockDim.x particles per CTA, or, persistent (an unstaged
    // launch of at most one resident wave: SimConsts::scan_persist), every
    // gridDim.x-th tile from blockIdx.x on
    if constexpr (Persist) {
        for (int i0 = blockIdx.x * blockDim.x; i0 < C.n; i0 += gridDim.x * blockDim.x)
            k_post_b_tile<Split, Stage>(C, P, V, Om, Nm, off, Vout, i0);
    } else {
        k_post_b_tile<Split, Stage>(C, P, V, Om, Nm, off, Vout, blockIdx.x * blockDim.x);
    }
}

// Pass C: XSPH viscosity (fluidXSph): same phase, j != i, r^2 <= h^2 (r = 0
// included).  Textbook mode weights each neighbour by its volume m_j / rho_j.
template <bool Split, bool Stage>
__device__ __forceinline__ void k_post_c_tile(
    const SimConsts &C,
    const float4 *__restrict__ P,
    const float4 *__restrict__ V,
    const int *__restrict__ off,
    const float *__restrict__ mass,
    const float *__restrict__ rho,
    float4 *__restrict__ Vout,
    int i0)
{
    StageShared &S = stage_shared();
    const int t = i0 + threadIdx.x;
    const int i = (Stage || t >= C.n) ? t : walker_index(C, t);
    const int cnt = post_list_count(C, P, i, t);
    const int g = (Stage && __syncthreads_or(cnt == kWalkCells)) ? stage_block(C, P, off, i0, S) : -1;
    if (i >= C.n) return;
    const float4 pi4 = P[i];
    const float4 vi4 = V[i];
    const int phi = phase_of(pi4);
    if (phi >= 0) {
        Vout[i] = vi4;
        return;
    }
    const float3 pi = f3(pi4), vi = f3(vi4);
    float3 vn = make_float3(0.f, 0.f, 0.f);
    auto body_at = [&](const float4 *__restrict__ Vp, const float *__restrict__ mp, const float *__restrict__ rp,
                       int j, float4 pj4) {
        float wgt = poly6(C, len2(pi - f3(pj4)));
        if (C.textbook) wgt = __fmul_rn(wgt, __fdiv_rn(__ldg(mp + j), __ldg(rp + j)));
        vn = fma3(wgt, f3(Vp[j]) - vi, vn);
    };
    auto body = [&](int j, float4 pj4) { body_at(V, mass, rho, j, pj4); };
    auto test = [&](int j, float4 pj4) { return j != i && phase_of(pj4) == phi && len2(pi - f3(pj4)) <= C.h2; };
    const GridView gv = grid_view(C, scene_index(C, i), off);
    int own = -1;
    // reference mode: each entry's velocity loads with its position, before
    // the four pair terms of a record
    auto listed = [&](int, float4 pj4, float4 vj4) { vn = fma3(poly6(C, len2(pi - f3(pj4))), f3(vj4) - vi, vn); };
    if (cnt != kWalkCells && post_slots(C, Stage) && !C.textbook) {  // V: pass B's output, in class order
        for_each_in_list_with(C.nbr, C.n, t, cnt, C.cls_pos, [&](int q) { return C.cls_vb[q]; }, listed);
    } else if (cnt != kWalkCells && !C.textbook) {
        for_each_in_list_with(C.nbr, C.n, t, cnt, P, [&](int j) { return V[j]; }, listed);
    } else if (cnt != kWalkCells && post_slots(C, Stage)) {
        for_each_in_list(C.nbr, C.n, t, cnt, C.cls_pos,
                         [&](int q, float4 pj4) { body_at(C.cls_vb, C.cls_mass, C.cls_rho, q, pj4); });
    } else if (cnt != kWalkCells) {
        for_each_in_list(C.nbr, C.n, t, cnt, P, body);
    } else if (C.nbr && !C.nbr_count) {
        // no pass A before it: record the walk's pairs, then sum over them
        ListWriter list(C.nbr, C.nbr_cap, C.n, t);
        walk_neighbors<Split>(i, pi, 0, P, gv, C, Stage ? &S : nullptr, g, test, [&](int j, float4) { list.push(j); });
        own = list.finish();
        if (own >= 0) for_each_in_list<false>(C.nbr, C.n, t, own, P, body);
    }
    if (cnt == kWalkCells && own < 0) walk_neighbors<Split>(i, pi, 0, P, gv, C, Stage ? &S : nullptr, g, test, body);
    const float3 v = vi + C.xsph_c * vn;
    Vout[i] = make_float4(v.x, v.y, v.z, vi4.w);
}

template <bool Split, bool Stage, bool Persist = false>
__global__ void __launch_bounds__(kScanThreads, BP_POSTBC_MIN_BLOCKS) k_post_c(
    SimConsts C,
    const float4 *__restrict__ P,
    const float4 *__restrict__ V,
    const int *__restrict__ off,
    const float *__restrict__ mass,
    const float *__restrict__ rho,
    float4 *__restrict__ Vout)
{
    // one tile of blockDim.x particles per CTA, or, persistent (an unstaged
    // launch of at most one resident wave: SimConsts::scan_persist), every
    // gridDim.x-th tile from blockIdx.x on
    if constexpr (Persist) {
        for (int i0 = blockIdx.x * blockDim.x; i0 < C.n; i0 += gridDim.x * blockDim.x)
            k_post_c_tile<Split, Stage>(C, P, V, off, mass, rho, Vout, i0);
    } else {
        k_post_c_tile<Split, Stage>(C, P, V, off, mass, rho, Vout, blockIdx.x * blockDim.x);
    }
}

void launch_post_a(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *V, const float *rho,
                   const int *off, float4 *Om, float4 *Nm, LaunchLog *L)
{
    if (C.n <= 0) return;
    BP_LAUNCH_SPLIT(k_post_a, st, C, P, V, rho, off, Om, Nm);
    L->done(__func__);
}
void launch_post_b(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *V, const float4 *Om,
                   const float4 *Nm, const int *off, float4 *Vout, LaunchLog *L)
{
    if (C.n <= 0) return;
    BP_LAUNCH_SPLIT(k_post_b, st, C, P, V, Om, Nm, off, Vout);
    L->done(__func__);
}
void launch_post_c(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *V, const int *off,
                   const float *mass, const float *rho, float4 *Vout, LaunchLog *L)
{
    if (C.n <= 0) return;
    BP_LAUNCH_SPLIT(k_post_c, st, C, P, V, off, mass, rho, Vout);
    L->done(__func__);
}

// Same count on caller buffers in the reference's start/end format.
__global__ void k_neighbor_counts_f3(int n, const float *__restrict__ pos3, float cell, int D, float h2,
                                     const int *__restrict__ start, const int *__restrict__ end,
                                     int *__restrict__ counts)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 pi = make_float3(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]);
    const unsigned m = (unsigned)D - 1u;
    const int cx = cell_coord(pi.x, cell), cy = cell_coord(pi.y, cell), cz = cell_coord(pi.z, cell);
    int cnt = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int a = cell_addr(cx + dx, cy + dy, cz + dz, D, m);
                const int b = start[a], e = end[a];
                for (int j = b; j < e; ++j) {
                    const float3 pj = make_float3(pos3[3 * j], pos3[3 * j + 1], pos3[3 * j + 2]);
                    if (len2(pi - pj) <= h2) ++cnt;
                }
            }
    counts[i] = cnt;
}

void launch_neighbor_counts_f3(cudaStream_t st, int n, const float *pos3, float cell, int D, float h,
                               const int *start, const int *end, int *counts)
{
    if (n <= 0) return;
    k_neighbor_counts_f3<<<(n + 127) / 128, 128, 0, st>>>(n, pos3, cell, D, h * h, start, end, counts);
}

}  // namespace bp
