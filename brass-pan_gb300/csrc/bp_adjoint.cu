// bp_adjoint.cu -- adjoint (reverse-mode) kernels of the substep stages.
//
// Each kernel takes the gradient of a scalar loss with respect to a stage's
// output and returns the gradient with respect to the stage's inputs (and
// parameters), given the stage's forward inputs as recorded by a re-run of
// that substep.  Pair and constraint sums are gathered per particle in a
// fixed order, as in the forward kernels, so gradients are deterministic.
// The neighbour sets are those of the forward pass (the same cell walk on
// the same positions).
//
// Supported stages: prediction and reorder, planes (stabilisation and
// collision), wind, particle-particle contacts with friction, fluid density /
// lambda / position correction in both modes (with s_corr and the per-pair
// clamp), distance constraints, dihedral bending, shape matching (rotation
// differentiated at its fixed point), immovables, the velocity update,
// vorticity confinement, Akinci tension, XSPH and picking.
#include <algorithm>

#include "bp_dual.cuh"
#include "bp_internal.h"
#include "bp_walk.cuh"

namespace bp {

__device__ __forceinline__ float3 ld3(const float4 *a, int i) { return f3(a[i]); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 mul3(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dotf(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float4 f4(float3 a, float w = 0.f) { return make_float4(a.x, a.y, a.z, w); }

// ---- planes, restated on dual numbers (plane_stabilize_with / plane_collide_with) ----

template <int N, class Planes>
__device__ void dplane_stabilize(const SimConsts &C, int np, Planes planes, V3<Dual<N>> &x, V3<Dual<N>> &p)
{
    for (int k = 0; k < np; ++k) {
        float3 o, n;
        planes(k, o, n);
        const Dual<N> d = dot(dv3<N>(o) - x, n) + C.radius;
        if (d.v <= 0.f) continue;
        x = x + scale_v(d, n);
        p = p + scale_v(d, n);
    }
}

template <int N, class Planes>
__device__ void dplane_collide(const SimConsts &C, int np, Planes planes, const V3<Dual<N>> &x, V3<Dual<N>> &p)
{
    for (int k = 0; k < np; ++k) {
        float3 o, n;
        planes(k, o, n);
        const Dual<N> d = dot(dv3<N>(o) - p, n) + C.radius;
        if (d.v <= 0.f) continue;
        const V3<Dual<N>> diff = p - x;
        const Dual<N> dn = dot(diff, n);
        const V3<Dual<N>> dt = diff - scale_v(dn, n);
        const Dual<N> dtl = dsqrt(dot(dt, dt));
        const V3<Dual<N>> resolved = scale_v(d, n) + p;
        const V3<Dual<N>> dx = resolved - x;
        const V3<Dual<N>> tdx = dx - scale_v(dot(dx, n), n);
        if (dtl.v < C.fs * dn.v)
            p = resolved - tdx;
        else
            p = resolved - scale(tdx, dmin((C.fd * -dn) / dtl, 1.0f));
    }
}

// Planes of scene s (s < 0: the solver's one scene) as the accessor above wants.
#define BP_PLANES_OF(C, s, body)                                                                      \
    do {                                                                                              \
        if ((s) < 0) {                                                                                \
            auto planes = [&](int k, float3 &o, float3 &n) { o = f3((C).plane_o[k]); n = f3((C).plane_n[k]); }; \
            const int np = (C).nplanes;                                                               \
            body;                                                                                     \
        } else {                                                                                      \
            const SceneConsts &Sc = (C).scn[s];                                                       \
            auto planes = [&](int k, float3 &o, float3 &n) { o = f3(Sc.plane_o[k]); n = f3(Sc.plane_n[k]); }; \
            const int np = Sc.nplanes;                                                                \
            body;                                                                                     \
        }                                                                                             \
    } while (0)

// ---- reorder: gather, predict, inverse scaled mass, 2x stabilise ----

__global__ void k_adj_reorder(SimConsts C, const int *__restrict__ order, const float4 *__restrict__ Xprev,
                              const float4 *__restrict__ Vprev, int stabilize, int inv_scaled,
                              const float4 *__restrict__ gP, const float4 *__restrict__ gXs,
                              const float4 *__restrict__ gVs, const float *__restrict__ gW,
                              float4 *__restrict__ gXprev, float4 *__restrict__ gVprev)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C.n) return;
    const int o = order[i];
    const float4 X = Xprev[o], V = Vprev[o];
    const int s = scene_index(C, i);
    const float3 gr = gravity_of(C, s);
    V3<Dual<6>> x = dv3var<6>(f3(X), 0), v = dv3var<6>(f3(V), 3);
    const float g2 = C.dt * C.dt;
    V3<Dual<6>> p = x + scale(v, C.dt);
    p = p + V3<Dual<6>>{dconst<6>(gr.x * g2), dconst<6>(gr.y * g2), dconst<6>(gr.z * g2)};
    if (stabilize) {
        BP_PLANES_OF(C, s, dplane_stabilize<6>(C, np, planes, x, p));
        BP_PLANES_OF(C, s, dplane_stabilize<6>(C, np, planes, x, p));
    }
    const float3 gp = f3(gP[i]), gx = f3(gXs[i]);
    float out[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) out[k] = vjp(p, gp, k) + vjp(x, gx, k);
    float3 gxo = make_float3(out[0], out[1], out[2]);
    float3 gvo = add3(make_float3(out[3], out[4], out[5]), f3(gVs[i]));
    if (inv_scaled) {  // w = 1 / (exp(-k y) m) = exp(k y) / m, dw/dy = k w
        const float w = 1.0f / (powf(2.7182818284f, -C.mass_k * X.y) * X.w);
        gxo.y += gW[i] * C.mass_k * w;
    }
    gXprev[o] = f4(gxo);
    gVprev[o] = f4(gvo);
}

// ---- planes (collision of predicted positions against the walls) ----

__global__ void k_adj_planes(SimConsts C, const float4 *__restrict__ Xs, const float4 *__restrict__ Pin,
                             float4 *__restrict__ gP, float4 *__restrict__ gXs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C.n) return;
    const int s = scene_index(C, i);
    const V3<Dual<6>> x = dv3var<6>(f3(Xs[i]), 0);
    V3<Dual<6>> p = dv3var<6>(f3(Pin[i]), 3);
    BP_PLANES_OF(C, s, dplane_collide<6>(C, np, planes, x, p));
    const float3 g = f3(gP[i]);
    const float4 gx = gXs[i];
    gXs[i] = make_float4(gx.x + vjp(p, g, 0), gx.y + vjp(p, g, 1), gx.z + vjp(p, g, 2), 0.f);
    gP[i] = make_float4(vjp(p, g, 3), vjp(p, g, 4), vjp(p, g, 5), 0.f);
}

// ---- velocity update and commit: x' = p, v' = (p - xs) / dt ----

__global__ void k_adj_commit(int n, float inv_dt, const float4 *__restrict__ gX, const float4 *__restrict__ gV,
                             float4 *__restrict__ gP, float4 *__restrict__ gXs, float4 *__restrict__ gVs,
                             float *__restrict__ gW)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 gv = mul3(f3(gV[i]), inv_dt);
    gP[i] = f4(add3(f3(gX[i]), gv));
    gXs[i] = f4(mul3(gv, -1.f));
    gVs[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    gW[i] = 0.f;
}

// ---- immovables: p = xs ----

__global__ void k_adj_immovable(int k, const int *__restrict__ ids, const int *__restrict__ to_new,
                                float4 *__restrict__ gP, float4 *__restrict__ gXs)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= k) return;
    const int i = to_new[ids[t]];
    gXs[i] = f4(add3(f3(gXs[i]), f3(gP[i])));
    gP[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ---- distance constraints ----
// Forward: x12 = p1 - p2, d = |x12|, k = n (d - L) / (w1 + w2) * s;
// p1 -= w1 k, p2 += w2 k.  Per edge: the gradient contributions to both
// endpoints (xyz: position, w: inverse scaled mass) and to s and L.

__global__ void k_adj_distance_edges(int m, const int2 *__restrict__ pairs, const float2 *__restrict__ params,
                                     const float4 *__restrict__ Pin, const float *__restrict__ w,
                                     const int *__restrict__ to_new, const float4 *__restrict__ gOut,
                                     float4 *__restrict__ G1, float4 *__restrict__ G2, float *__restrict__ g_stiff,
                                     float *__restrict__ g_rest)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    const int2 pr = pairs[e];
    const float2 prm = params[e];
    const int id1 = to_new[pr.x], id2 = to_new[pr.y];
    const float3 x12 = sub3(ld3(Pin, id1), ld3(Pin, id2));
    const float d = sqrtf(dotf(x12, x12));
    if (d <= 1e-5f) {
        G1[e] = make_float4(0.f, 0.f, 0.f, 0.f);
        G2[e] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float w1 = w[id1], w2 = w[id2], sw = w1 + w2;
    const float3 n = mul3(x12, 1.0f / d);
    const float sc = (d - prm.x) / sw * prm.y;
    const float3 k = mul3(n, sc);
    const float3 g1 = ld3(gOut, id1), g2 = ld3(gOut, id2);
    const float3 kb = add3(mul3(g1, -w1), mul3(g2, w2));
    float wb1 = -dotf(k, g1), wb2 = dotf(k, g2);
    const float3 nb = mul3(kb, sc);
    const float sb = dotf(kb, n);
    const float db = sb * prm.y / sw;
    const float swb = -sb * (d - prm.x) * prm.y / (sw * sw);
    wb1 += swb;
    wb2 += swb;
    const float3 xb = add3(mul3(sub3(nb, mul3(n, dotf(n, nb))), 1.0f / d), mul3(n, db));
    G1[e] = f4(xb, wb1);
    G2[e] = f4(mul3(xb, -1.f), wb2);
    g_stiff[e] += sb * (d - prm.x) / sw;
    g_rest[e] += -sb * prm.y / sw;
}

__global__ void k_adj_distance_apply(int nn_, const int *__restrict__ node_ids, const int *__restrict__ ptr,
                                     const int *__restrict__ inc, const float4 *__restrict__ G1,
                                     const float4 *__restrict__ G2, const int *__restrict__ to_new,
                                     float4 *__restrict__ gP, float *__restrict__ gW)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn_) return;
    const int i = to_new[node_ids[t]];
    float3 g = f3(gP[i]);
    float gw = gW[i];
    for (int q = ptr[t]; q < ptr[t + 1]; ++q) {
        const int code = inc[q];
        const float4 c = (code & 1) ? G2[code >> 1] : G1[code >> 1];
        g = add3(g, f3(c));
        gw += c.w;
    }
    gP[i] = f4(g);
    gW[i] = gw;
}

// ---- wind (per triangle: drag and lift from the face velocity) ----

template <int N>
__device__ V3<Dual<N>> wind_move(const SimConsts &C, const V3<Dual<N>> &a, const V3<Dual<N>> &b,
                                 const V3<Dual<N>> &v)
{
    V3<Dual<N>> mv = dv3<N>(make_float3(0.f, 0.f, 0.f));
    const Dual<N> lv = dsqrt(dot(v, v));
    if (lv.v <= 1e-5f) return mv;
    const V3<Dual<N>> vh = scale(v, dconst<N>(1.f) / lv);
    V3<Dual<N>> fn = cross(a, b);
    const Dual<N> lf = dsqrt(dot(fn, fn));
    if (lf.v <= 1e-5f) return mv;
    fn = scale(fn, dconst<N>(1.f) / lf);
    if (!(dot(fn, v).v > 0.f)) fn = -fn;
    const Dual<N> area = lf * 0.5f;
    const Dual<N> lv2 = lv * lv;
    const Dual<N> fv = dot(fn, vh);
    const V3<Dual<N>> drag = scale(-vh, (C.wind_drag * lv2) * area * fv);
    const V3<Dual<N>> uh = cross(cross(fn, vh), vh);
    const V3<Dual<N>> lift = scale(uh, (C.wind_lift * lv2) * area * fv);
    return scale(drag + lift, C.dt * C.dt);
}

__global__ void k_adj_wind_faces(SimConsts C, int nf, const int *__restrict__ faces, const float4 *__restrict__ Pin,
                                 const float4 *__restrict__ Vs, const float *__restrict__ mass,
                                 const int *__restrict__ to_new, const float4 *__restrict__ gOut,
                                 float4 *__restrict__ FG, float4 *__restrict__ FV, float4 *__restrict__ FW)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int i1 = to_new[faces[3 * f]], i2 = to_new[faces[3 * f + 1]], i3 = to_new[faces[3 * f + 2]];
    const float3 p1 = ld3(Pin, i1), p2 = ld3(Pin, i2), p3 = ld3(Pin, i3);
    float3 v = mul3(add3(add3(ld3(Vs, i1), ld3(Vs, i2)), ld3(Vs, i3)), 1.0f / 3.0f);
    if (C.textbook) v = sub3(v, C.wind);
    const V3<Dual<9>> mv = wind_move<9>(C, dv3var<9>(sub3(p2, p1), 0), dv3var<9>(sub3(p3, p1), 3), dv3var<9>(v, 6));
    const float3 g = add3(add3(mul3(ld3(gOut, i1), 1.0f / mass[i1]), mul3(ld3(gOut, i2), 1.0f / mass[i2])),
                          mul3(ld3(gOut, i3), 1.0f / mass[i3]));
    const float3 ab = make_float3(vjp(mv, g, 0), vjp(mv, g, 1), vjp(mv, g, 2));
    const float3 bb = make_float3(vjp(mv, g, 3), vjp(mv, g, 4), vjp(mv, g, 5));
    const float3 vb = make_float3(vjp(mv, g, 6), vjp(mv, g, 7), vjp(mv, g, 8));
    FG[3 * f] = f4(mul3(add3(ab, bb), -1.f));
    FG[3 * f + 1] = f4(ab);
    FG[3 * f + 2] = f4(bb);
    FV[f] = f4(mul3(vb, 1.0f / 3.0f));
    FW[f] = C.textbook ? f4(mul3(vb, -1.f)) : make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void k_adj_wind_apply(int nn_, const int *__restrict__ node_ids, const int *__restrict__ ptr,
                                 const int *__restrict__ inc, const int *__restrict__ faces,
                                 const float4 *__restrict__ FG, const float4 *__restrict__ FV,
                                 const int *__restrict__ to_new, float4 *__restrict__ gP, float4 *__restrict__ gVs)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn_) return;
    const int id = node_ids[t];
    const int i = to_new[id];
    float3 g = f3(gP[i]), gv = f3(gVs[i]);
    for (int q = ptr[t]; q < ptr[t + 1]; ++q) {
        const int f = inc[q];
        const int corner = faces[3 * f] == id ? 0 : (faces[3 * f + 1] == id ? 1 : 2);
        g = add3(g, f3(FG[3 * f + corner]));
        gv = add3(gv, f3(FV[f]));
    }
    gP[i] = f4(g);
    gVs[i] = f4(gv);
}

// Deterministic sum of n float4 into acc (one CTA, fixed partition and tree).
__global__ void __launch_bounds__(1024) k_adj_sum4(int n, const float4 *__restrict__ a, float4 *__restrict__ acc)
{
    __shared__ float4 red[1024];
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = threadIdx.x; k < n; k += 1024) {
        const float4 v = a[k];
        s.x += v.x;
        s.y += v.y;
        s.z += v.z;
        s.w += v.w;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = 512; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            const float4 o = red[threadIdx.x + h];
            red[threadIdx.x].x += o.x;
            red[threadIdx.x].y += o.y;
            red[threadIdx.x].z += o.z;
            red[threadIdx.x].w += o.w;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        acc->x += red[0].x;
        acc->y += red[0].y;
        acc->z += red[0].z;
        acc->w += red[0].w;
    }
}

// ---- fluid, reference mode ----
// rho_i = sum_{j >= i, r <= h} m_j s_j W6(r_ij); lambda_i = -max(C_i, 0 if Akinci) / den
// dp_i = (1/rho0) sum_j m_j clamp((lambda_i + lambda_j - scorr(r_ij)) gradW(r_ij))

struct SpikyD {
    float3 g;    // grad W(r)
    float f, fp; // grad W = f(|r|) r, f' = df/d|r|
};
__device__ __forceinline__ SpikyD spiky_d(const SimConsts &C, float3 r, float rl)
{
    SpikyD s;
    const float t = C.h - rl;
    s.f = C.c_spiky * t * t / rl;
    s.fp = C.c_spiky * (-2.f * t / rl - t * t / (rl * rl));
    s.g = mul3(r, s.f);
    return s;
}
// H(r) u for the spiky gradient's Jacobian H = f I + f' r r^T / |r|
__device__ __forceinline__ float3 spiky_hess_mul(const SpikyD &s, float3 r, float rl, float3 u)
{
    return add3(mul3(u, s.f), mul3(r, s.fp * dotf(r, u) / rl));
}
__device__ __forceinline__ float3 poly6_grad(const SimConsts &C, float3 r, float r2)
{
    const float t = C.h2 - r2;
    return mul3(r, -6.f * C.c_poly6 * t * t);
}
// J^T g of the per-pair clamp u -> u (|u| < c) or c u / |u|
__device__ __forceinline__ float3 clamp_vjp(const SimConsts &C, float3 u, float3 g)
{
    if (!(C.delta_clamp > 0.f)) return g;
    const float l2 = dotf(u, u);
    if (l2 < C.delta_clamp2) return g;
    const float l = sqrtf(l2);
    const float3 uh = mul3(u, 1.0f / l);
    return mul3(sub3(g, mul3(uh, dotf(uh, g))), C.delta_clamp / l);
}
__device__ __forceinline__ float3 clamp_fwd(const SimConsts &C, float3 u)
{
    if (!(C.delta_clamp > 0.f)) return u;
    const float l2 = dotf(u, u);
    if (l2 < C.delta_clamp2) return u;
    return mul3(u, C.delta_clamp / sqrtf(l2));
}

// The pairs of particle k that pass test, in walk order: term(j, P[j],
// fetch(j)).  With C.nbr the walk records the pairs that pass `record` (a
// superset of test's) and the terms of those that pass test are summed over
// the list, each record's four positions and fetch() data loaded before its
// four terms; the list's count goes to C.nbr_count[k] (-1: overflow), so that
// a later pass over the same positions can read it.  Without lists, or past
// the list's capacity, the terms run inside the walk.
template <class R, class T, class G, class B>
__device__ __forceinline__ void record_then_sum(const SimConsts &C, int k, float3 pk, const float4 *__restrict__ P,
                                                const GridView &v, const StageShared *S, int g, R &record, T &test,
                                                G &fetch, B &term)
{
    int cnt = -1;
    if (C.nbr) {
        ListWriter list(C.nbr, C.nbr_cap, C.n, k);
        walk_neighbors<true>(k, pk, 0, P, v, C, S, g, record, [&](int j, float4) { list.push(j); });
        cnt = list.finish();
        if (C.nbr_count) C.nbr_count[k] = cnt;
        if (cnt >= 0)
            for_each_in_list_with<false>(C.nbr, C.n, k, cnt, P, fetch, [&](int j, float4 pj, const auto &nb) {
                if (test(j, pj)) term(j, pj, nb);
            });
    }
    if (cnt < 0) walk_neighbors<true>(k, pk, 0, P, v, C, S, g, test, [&](int j, float4 pj) { term(j, pj, fetch(j)); });
}
// The same with no per-neighbour data: term(j, P[j]).
template <class R, class T, class B>
__device__ __forceinline__ void record_then_sum(const SimConsts &C, int k, float3 pk, const float4 *__restrict__ P,
                                                const GridView &v, const StageShared *S, int g, R &record, T &test,
                                                B &term)
{
    auto none = [](int) { return 0; };
    auto term3 = [&](int j, float4 pj, int) { term(j, pj); };
    record_then_sum(C, k, pk, P, v, S, g, record, test, none, term3);
}

// Walk A: lambda-bar and the position gradient of the correction terms.  It
// records every j != k within h (the pairs of the density terms, a superset
// of its own), so that pass B sums over the same list instead of walking.
__global__ void __launch_bounds__(kWalkThreads) k_adj_deltap(SimConsts C, const float4 *__restrict__ P,
                                                             const float *__restrict__ mass,
                                                             const float *__restrict__ lam, const int *__restrict__ off,
                                                             const float4 *__restrict__ gOut,
                                                             float *__restrict__ gLam, float4 *__restrict__ gPart)
{
    StageShared &S = stage_shared();
    const int g = stage_block(C, P, off, blockIdx.x * kWalkThreads, S);
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= C.n) return;
    const float4 pk4 = P[k];
    const int phk = phase_of(pk4);
    const float3 pk = f3(pk4);
    const int sc = scene_index(C, k);
    const float inv_rho0 = inv_rest_density(C, sc);
    const float lk = lam[k], mk = mass[k];
    const float3 gk = ld3(gOut, k);
    float lb = 0.f;
    float3 pb = make_float3(0.f, 0.f, 0.f);
    // reference mode: the pair counts for both ends when its lower index is
    // fluid; textbook mode: every fluid particle gathers over all neighbours
    auto test = [&](int j, float4 pj4) {
        const float3 r = sub3(pk, f3(pj4));
        const float d2 = dotf(r, r);
        const bool fj = phase_of(pj4) < 0;
        const bool inc = C.textbook ? (phk < 0 || fj) : ((j > k) ? (phk < 0) : fj);
        return j != k && d2 <= C.h2 && d2 > 0.f && inc;
    };
    // a neighbour's lambda, mass and incoming gradient
    struct Nb {
        float lam, mass;
        float4 g;
    };
    auto fetch = [&](int j) { return Nb{__ldg(lam + j), __ldg(mass + j), gOut[j]}; };
    auto term = [&](int j, float4 pj4, const Nb &nb) {
            const float3 r = sub3(pk, f3(pj4));
            const float d2 = dotf(r, r);
            const float rl = sqrtf(d2);
            const bool own = !C.textbook || phk < 0;               // dp_k has the pair
            const bool other = !C.textbook || phase_of(pj4) < 0;  // dp_j has the pair
            const SpikyD sp = spiky_d(C, r, rl);
            float s = lk + nb.lam;
            float3 dsc = make_float3(0.f, 0.f, 0.f);  // d scorr / d r
            if (C.scorr_on) {
                const float x = poly6(C, d2) * C.scorr_inv_wq;
                s -= C.scorr_k * ipowf(x, C.scorr_ni);
                if (C.scorr_ni > 0)
                    dsc = mul3(poly6_grad(C, r, d2), C.scorr_k * C.scorr_ni * ipowf(x, C.scorr_ni - 1) * C.scorr_inv_wq);
            }
            // term of dp_k: (m_j / rho0) clamp(s gradW(r))
            const float3 u1b = own ? mul3(clamp_vjp(C, mul3(sp.g, s), gk), nb.mass * inv_rho0)
                                   : make_float3(0.f, 0.f, 0.f);
            const float sb1 = dotf(u1b, sp.g);
            const float3 rb1 = sub3(mul3(spiky_hess_mul(sp, r, rl, u1b), s), mul3(dsc, sb1));
            // term of dp_j: (m_k / rho0) clamp(s gradW(-r))
            const float3 g_neg = mul3(sp.g, -1.f);
            const float3 u2b = other ? mul3(clamp_vjp(C, mul3(g_neg, s), f3(nb.g)), mk * inv_rho0)
                                     : make_float3(0.f, 0.f, 0.f);
            const float sb2 = dotf(u2b, g_neg);
            // gradient w.r.t. r_jk = -r: H(-r) = H(r), dscorr(-r) = -dscorr(r)
            const float3 rb2 = add3(mul3(spiky_hess_mul(sp, r, rl, u2b), s), mul3(dsc, sb2));
            lb += sb1 + sb2;
            pb = add3(pb, sub3(rb1, rb2));
    };
    auto within = [&](int j, float4 pj4) {
        const float3 r = sub3(pk, f3(pj4));
        return j != k && dotf(r, r) <= C.h2;
    };
    record_then_sum(C, k, pk, P, grid_view(C, sc, off), &S, g, within, test, fetch, term);
    gLam[k] = lb;
    gPart[k] = f4(pb);
}

// Pass B: the density gradient; gP (in) = gOut + gPart + density terms.  It
// sums over the list pass A recorded at the same positions (every j != k
// within h, in walk order) and walks only where that list overflowed.
__global__ void __launch_bounds__(kWalkThreads, 3) k_adj_lambda(SimConsts C, const float4 *__restrict__ P,
                                                             const float *__restrict__ mass,
                                                             const float *__restrict__ rho, const int *__restrict__ off,
                                                             const float *__restrict__ gLam,
                                                             const float4 *__restrict__ gPart,
                                                             const float4 *__restrict__ gOut,
                                                             const float *__restrict__ gRho, float4 *__restrict__ gIn)
{
    StageShared &S = stage_shared();
    const int g = stage_block(C, P, off, blockIdx.x * kWalkThreads, S);
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= C.n) return;
    const float4 pk4 = P[k];
    const int phk = phase_of(pk4);
    const float3 pk = f3(pk4);
    const int sc = scene_index(C, k);
    const float rho0 = rest_density(C, sc);
    auto rho_bar = [&](int j, int phj) {
        if (phj > 0) return 0.f;  // solids: lambda is 0 whatever the density
        const float ext = gRho ? gRho[j] : 0.f;  // the density's gradient through the post passes
        if (C.clamp_c && !(rho[j] / rho0 - 1.0f > 0.f)) return ext;
        return ext - gLam[j] / (C.lambda_den * rho0);
    };
    const float rbk = rho_bar(k, phk);
    const float mk = mass[k] * (phk < 0 ? 1.f : C.solid_scale);
    float3 pb = make_float3(0.f, 0.f, 0.f);
    auto test = [&](int j, float4 pj4) { return j != k && dotf(sub3(pk, f3(pj4)), sub3(pk, f3(pj4))) <= C.h2; };
    // what rho_bar and the term read of a neighbour, loaded with its position
    struct Nb {
        float gl, gr, rh, m;
    };
    auto fetch = [&](int j) { return Nb{gLam[j], gRho ? gRho[j] : 0.f, rho[j], mass[j]}; };
    auto term = [&](int j, float4 pj4, const Nb &nb) {
        const int phj = phase_of(pj4);
        const float3 r = sub3(pk, f3(pj4));
        const float3 gw = poly6_grad(C, r, dotf(r, r));
        if (j > k) {
            pb = add3(pb, mul3(gw, rbk * nb.m * (phj < 0 ? 1.f : C.solid_scale)));
        } else {
            // rho_bar(j, phj) from the loaded values
            float rb = 0.f;
            if (phj <= 0) rb = (C.clamp_c && !(nb.rh / rho0 - 1.0f > 0.f)) ? nb.gr : nb.gr - nb.gl / (C.lambda_den * rho0);
            pb = add3(pb, mul3(gw, rb * mk));
        }
    };
    const int cnt = (C.nbr && C.nbr_count) ? __ldg(C.nbr_count + k) : -1;
    if (cnt >= 0)  // pass A's list: exactly test's pairs
        for_each_in_list_with(C.nbr, C.n, k, cnt, P, fetch, term);
    else
        walk_neighbors<true>(k, pk, 0, P, grid_view(C, sc, off), C, &S, g, test,
                             [&](int j, float4 pj4) { term(j, pj4, fetch(j)); });
    gIn[k] = f4(add3(add3(ld3(gOut, k), ld3(gPart, k)), pb));
}

// ---- fluid, textbook mode ----
// rho_i = sum_j m_j s_j W6(r_ij) (all j, the particle itself included),
// G_i = sum_{j != i} a_j gradW(r_ij), a_j = m_j / rho0,
// D_i = sum_{j != i} a_j^2 |gradW(r_ij)|^2 + |G_i|^2 + eps, lambda_i = -C_i / D_i;
// dp_k as in reference mode for every fluid k over all its neighbours.
// Pass T2 turns lambda-bar into rho-bar and D-bar per fluid particle; pass T3
// gathers their position terms: as particle i of its own sums and as
// neighbour j of its neighbours' sums.

__global__ void __launch_bounds__(kWalkThreads) k_adj_lambda_tb_prep(SimConsts C, const float4 *__restrict__ P,
                                                                     const float *__restrict__ mass,
                                                                     const int *__restrict__ off,
                                                                     const float *__restrict__ gLam,
                                                                     const float *__restrict__ gRho,
                                                                     float4 *__restrict__ GD, float *__restrict__ rhob)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= C.n) return;
    const float4 pk4 = P[k];
    if (phase_of(pk4) > 0) {  // solids: lambda 0 whatever their neighbours
        GD[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        rhob[k] = 0.f;
        return;
    }
    const float3 pk = f3(pk4);
    const int sc = scene_index(C, k);
    const float rho0 = rest_density(C, sc), inv_rho0 = 1.0f / rho0;
    float rho = 0.f, g2 = 0.f;
    float3 G = make_float3(0.f, 0.f, 0.f);
    auto test = [&](int, float4 pj4) { return dotf(sub3(pk, f3(pj4)), sub3(pk, f3(pj4))) <= C.h2; };
    auto term = [&](int j, float4 pj4) {
        const float3 r = sub3(pk, f3(pj4));
        const float d2 = dotf(r, r);
        const float ld = mass[j] * poly6(C, d2);
        rho += phase_of(pj4) < 0 ? ld : C.solid_scale * ld;
        if (d2 > 0.f) {
            const float3 g = mul3(spiky_d(C, r, sqrtf(d2)).g, mass[j] * inv_rho0);
            g2 += dotf(g, g);
            G = add3(G, g);
        }
    };
    walk_neighbors<true>(k, pk, 0, P, grid_view(C, sc, off), C, nullptr, -1, test, term);
    const float D = g2 + dotf(G, G) + C.relaxation;
    float c = rho / rho0 - 1.0f;
    const bool clamped = C.clamp_c && !(c > 0.f);
    if (clamped) c = 0.f;
    const float lb = gLam[k];
    const float cb = clamped ? 0.f : -lb / D;
    GD[k] = f4(G, lb * c / (D * D));
    rhob[k] = cb / rho0 + (gRho ? gRho[k] : 0.f);
}

__global__ void __launch_bounds__(kWalkThreads) k_adj_lambda_tb(SimConsts C, const float4 *__restrict__ P,
                                                                const float *__restrict__ mass,
                                                                const int *__restrict__ off,
                                                                const float4 *__restrict__ GD,
                                                                const float *__restrict__ rhob,
                                                                const float4 *__restrict__ gPart,
                                                                const float4 *__restrict__ gOut,
                                                                float4 *__restrict__ gIn)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= C.n) return;
    const float4 pk4 = P[k];
    const int phk = phase_of(pk4);
    const float3 pk = f3(pk4);
    const int sc = scene_index(C, k);
    const float inv_rho0 = inv_rest_density(C, sc);
    const float4 gdk = GD[k];
    const float3 Gk = f3(gdk);
    const float Dbk = gdk.w, rbk = rhob[k];
    const float mk = mass[k], ak = mk * inv_rho0, sk = phk < 0 ? 1.f : C.solid_scale;
    float3 pb = make_float3(0.f, 0.f, 0.f);
    auto test = [&](int j, float4 pj4) {
        const float3 r = sub3(pk, f3(pj4));
        const float d2 = dotf(r, r);
        return j != k && d2 <= C.h2 && d2 > 0.f;
    };
    auto term = [&](int j, float4 pj4) {
        const float3 r = sub3(pk, f3(pj4));
        const float d2 = dotf(r, r), rl = sqrtf(d2);
        const SpikyD sp = spiky_d(C, r, rl);
        const float3 w6 = poly6_grad(C, r, d2);
        const int phj = phase_of(pj4);
        const float mj = mass[j], aj = mj * inv_rho0;
        if (phk < 0) {  // k's own density and denominator
            const float3 u = mul3(add3(mul3(sp.g, 2.f * aj * aj), mul3(Gk, 2.f * aj)), Dbk);
            pb = add3(add3(pb, spiky_hess_mul(sp, r, rl, u)), mul3(w6, rbk * mj * (phj < 0 ? 1.f : C.solid_scale)));
        }
        if (phj < 0) {  // j's, through r_jk = -r
            const float4 gdj = GD[j];
            const float3 u = mul3(sub3(mul3(sp.g, 2.f * ak * ak), mul3(f3(gdj), 2.f * ak)), gdj.w);
            pb = add3(add3(pb, spiky_hess_mul(sp, r, rl, u)), mul3(w6, rhob[j] * mk * sk));
        }
    };
    walk_neighbors<true>(k, pk, 0, P, grid_view(C, sc, off), C, nullptr, -1, test, term);
    gIn[k] = f4(add3(add3(ld3(gOut, k), ld3(gPart, k)), pb));
}

// ---- XSPH: v'_i = v_i + c sum_j W6(r_ij) b_j (v_j - v_i) ----
// b_j = 1 in reference mode, m_j / rho_j in textbook mode (whose density
// gradient is added to gRho).  Positions are the committed ones; gX receives
// their gradient.

__global__ void __launch_bounds__(kWalkThreads) k_adj_xsph(SimConsts C, const float4 *__restrict__ P,
                                                           const float4 *__restrict__ V, const int *__restrict__ off,
                                                           const float *__restrict__ mass,
                                                           const float *__restrict__ rho,
                                                           const float4 *__restrict__ gVout, float4 *__restrict__ gVin,
                                                           float4 *__restrict__ gX, float *__restrict__ gRho)
{
    StageShared &S = stage_shared();
    const int g = stage_block(C, P, off, blockIdx.x * kWalkThreads, S);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C.n) return;
    const float4 pi4 = P[i];
    const int phi = phase_of(pi4);
    const float3 go = ld3(gVout, i);
    if (phi >= 0) {
        gVin[i] = f4(go);
        return;
    }
    const float3 pi = f3(pi4), vi = ld3(V, i);
    const float bi = C.textbook ? mass[i] / rho[i] : 1.f;
    float3 gv = go, gp = make_float3(0.f, 0.f, 0.f);
    float rb = 0.f;
    auto test = [&](int j, float4 pj4) {
        const float3 r = sub3(pi, f3(pj4));
        return j != i && phase_of(pj4) == phi && dotf(r, r) <= C.h2;
    };
    auto term = [&](int j, float4 pj4) {
        const float3 r = sub3(pi, f3(pj4));
        const float d2 = dotf(r, r);
        const float w = poly6(C, d2);
        const float bj = C.textbook ? mass[j] / rho[j] : 1.f;
        const float3 gj = ld3(gVout, j);
        gv = add3(gv, mul3(sub3(mul3(gj, bi), mul3(go, bj)), C.xsph_c * w));
        const float3 dv = sub3(ld3(V, j), vi);
        gp = add3(gp, mul3(poly6_grad(C, r, d2), C.xsph_c * (bj * dotf(dv, go) - bi * dotf(dv, gj))));
        if (C.textbook) rb -= C.xsph_c * w * dotf(dv, gj);  // j's sum: c W b_i (v_i - v_j) . g_j
    };
    record_then_sum(C, i, pi, P, grid_view(C, scene_index(C, i), off), &S, g, test, test, term);
    gVin[i] = f4(gv);
    gX[i] = f4(add3(ld3(gX, i), gp));
    if (C.textbook) gRho[i] -= rb * bi / rho[i];  // d b_i / d rho_i = -b_i / rho_i
}

// ---- shape matching (alpha = 1): g_i = R q_i + cm ----
// cm = mean(p_i), A = sum (p_i - cm) q_i^T, R the rotation the extraction
// converged to (recorded).  R is differentiated implicitly through its fixed
// point, where R^T A = S is symmetric: dR = R [w]x with (tr(S) I - S) w =
// vee(R^T dA - dA^T R).  Hence A-bar = R [z]x with z = (tr(S) I - S)^-1
// vee(R^T R-bar - R-bar^T R), R-bar = sum g-bar_i q_i^T.

struct M3 {
    float m[3][3];  // row-major
};
__device__ __forceinline__ M3 quat_mat(float4 q)
{
    const float x = q.x, y = q.y, z = q.z, w = q.w;
    M3 r;
    r.m[0][0] = 1 - 2 * y * y - 2 * z * z;
    r.m[1][0] = 2 * x * y + 2 * w * z;
    r.m[2][0] = 2 * x * z - 2 * w * y;
    r.m[0][1] = 2 * x * y - 2 * w * z;
    r.m[1][1] = 1 - 2 * x * x - 2 * z * z;
    r.m[2][1] = 2 * y * z + 2 * w * x;
    r.m[0][2] = 2 * x * z + 2 * w * y;
    r.m[1][2] = 2 * y * z - 2 * w * x;
    r.m[2][2] = 1 - 2 * x * x - 2 * y * y;
    return r;
}

constexpr int kAdjSmThreads = 256;

template <int NV>
__device__ __forceinline__ void adj_block_sum(float (&v)[NV], float (*red)[kAdjSmThreads / 32])
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
        for (int q = 0; q < kAdjSmThreads / 32; ++q) s += red[k][q];
        v[k] = s;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kAdjSmThreads) k_adj_shape_matching(RigidArgs a, const float4 *__restrict__ rotq,
                                                                      const float4 *__restrict__ Pin,
                                                                      const int *__restrict__ to_new,
                                                                      float4 *__restrict__ gP)
{
    __shared__ float red[12][kAdjSmThreads / 32];
    __shared__ float s_abar[9], s_cmb[3];
    const int b = blockIdx.x;
    const int2 rg = a.ranges[b];
    const int np = rg.y - rg.x;
    float c[3] = {0.f, 0.f, 0.f};
    for (int t = threadIdx.x; t < np; t += kAdjSmThreads) {
        const float3 p = ld3(Pin, to_new[rg.x + t]);
        c[0] += p.x;
        c[1] += p.y;
        c[2] += p.z;
    }
    adj_block_sum<3>(c, red);
    const float3 cm = make_float3(c[0] / np, c[1] / np, c[2] / np);
    // A (row-major), R-bar, sum of g-bar, sum of q
    float acc[12] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float acc2[12] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int t = threadIdx.x; t < np; t += kAdjSmThreads) {
        const int id = to_new[rg.x + t];
        const float3 q = f3(a.rest[rg.x + t]);
        const float3 pc = sub3(ld3(Pin, id), cm);
        const float3 g = ld3(gP, id);
        const float pv[3] = {pc.x, pc.y, pc.z}, qv[3] = {q.x, q.y, q.z}, gv[3] = {g.x, g.y, g.z};
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) {
                acc[3 * r + k] += pv[r] * qv[k];   // A
                acc2[3 * r + k] += gv[r] * qv[k];  // R-bar
            }
        acc[9] += g.x;
        acc[10] += g.y;
        acc[11] += g.z;
        acc2[9] += q.x;
        acc2[10] += q.y;
        acc2[11] += q.z;
    }
    adj_block_sum<12>(acc, red);
    adj_block_sum<12>(acc2, red);
    if (threadIdx.x == 0) {
        const M3 R = quat_mat(rotq[b]);
        float S[3][3], X[3][3];  // S = R^T A, X = R^T R-bar
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                float s = 0.f, x = 0.f;
                for (int k = 0; k < 3; ++k) {
                    s += R.m[k][i] * acc[3 * k + j];
                    x += R.m[k][i] * acc2[3 * k + j];
                }
                S[i][j] = s;
                X[i][j] = x;
            }
        const float u[3] = {X[2][1] - X[1][2], X[0][2] - X[2][0], X[1][0] - X[0][1]};
        const float tr = S[0][0] + S[1][1] + S[2][2];
        float G[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) G[i][j] = (i == j ? tr : 0.f) - 0.5f * (S[i][j] + S[j][i]);
        // z = G^-1 u by the adjugate
        const float c00 = G[1][1] * G[2][2] - G[1][2] * G[2][1], c01 = G[1][2] * G[2][0] - G[1][0] * G[2][2],
                    c02 = G[1][0] * G[2][1] - G[1][1] * G[2][0];
        const float det = G[0][0] * c00 + G[0][1] * c01 + G[0][2] * c02;
        float z[3] = {0.f, 0.f, 0.f};
        if (fabsf(det) > 1e-20f) {
            const float inv = 1.0f / det;
            const float Gi[3][3] = {{c00 * inv, (G[0][2] * G[2][1] - G[0][1] * G[2][2]) * inv,
                                     (G[0][1] * G[1][2] - G[0][2] * G[1][1]) * inv},
                                    {c01 * inv, (G[0][0] * G[2][2] - G[0][2] * G[2][0]) * inv,
                                     (G[0][2] * G[1][0] - G[0][0] * G[1][2]) * inv},
                                    {c02 * inv, (G[0][1] * G[2][0] - G[0][0] * G[2][1]) * inv,
                                     (G[0][0] * G[1][1] - G[0][1] * G[1][0]) * inv}};
            for (int i = 0; i < 3; ++i) z[i] = Gi[i][0] * u[0] + Gi[i][1] * u[1] + Gi[i][2] * u[2];
        }
        const float Z[3][3] = {{0.f, -z[2], z[1]}, {z[2], 0.f, -z[0]}, {-z[1], z[0], 0.f}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                s_abar[3 * i + j] = R.m[i][0] * Z[0][j] + R.m[i][1] * Z[1][j] + R.m[i][2] * Z[2][j];
        // cm-bar: from the goals (sum g-bar) and from A through p_i - cm (-A-bar sum q)
        for (int i = 0; i < 3; ++i)
            s_cmb[i] = acc[9 + i] - (s_abar[3 * i] * acc2[9] + s_abar[3 * i + 1] * acc2[10] + s_abar[3 * i + 2] * acc2[11]);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < np; t += kAdjSmThreads) {
        const int id = to_new[rg.x + t];
        const float3 q = f3(a.rest[rg.x + t]);
        float3 g;
        g.x = s_abar[0] * q.x + s_abar[1] * q.y + s_abar[2] * q.z + s_cmb[0] / np;
        g.y = s_abar[3] * q.x + s_abar[4] * q.y + s_abar[5] * q.z + s_cmb[1] / np;
        g.z = s_abar[6] * q.x + s_abar[7] * q.y + s_abar[8] * q.z + s_cmb[2] / np;
        gP[id] = f4(g);
    }
}

// ---- particle-particle contacts (collide_one, bp_constraints.cu) ----
// Only the mover i changes: p_i' = p_i + sum_j dx_ij + (1 / c_i) sum_{j counted}
// f_ij, where dx_ij is the mass-weighted projection of the pair, f_ij its
// friction move (from the substep-start positions Xs) and c_i the number of
// counted pairs of i (piecewise constant: no derivative).  Inputs of a pair:
// both predicted positions, both start positions, both inverse scaled masses.

// The pair filter of collide_one: different phases, one of them solid, closer
// than two radii and not coincident.
__device__ __forceinline__ bool contact_pair(const SimConsts &C, float3 pi, int phi, float4 pj4)
{
    const int phj = phase_of(pj4);
    const float d2 = len2(pi - f3(pj4));
    const float r = C.radius;
    return phi != phj && (phi > 0 || phj > 0) && d2 < r * r * 4.0f && d2 > 1e-5f;
}

// Does the pair count for friction (collide_one's test, in its float operations)?
__device__ __forceinline__ bool contact_counted(const SimConsts &C, float3 pi, float wi, float3 pj, float wj)
{
    const float r = C.radius;
    const float3 diff = pi - pj;
    const float dist = __fsqrt_rn(len2(diff));
    const float w1 = __fdiv_rn(wi, __fadd_rn(wi, wj));
    const float3 dxi = w1 * (diff * __fsub_rn(__fdiv_rn(2.0f * r, dist), 1.0f));
    return len2(dxi) > r * r * 0.001f * 0.001f;
}

// The move of mover i from partner j, on dual numbers; count: c_i.
template <int N>
__device__ __forceinline__ V3<Dual<N>> dcontact(const SimConsts &C, const V3<Dual<N>> &pi, const V3<Dual<N>> &xi,
                                const Dual<N> &wi, const V3<Dual<N>> &pj, const V3<Dual<N>> &xj,
                                const Dual<N> &wj, bool counted, int count)
{
    const float r = C.radius;
    const V3<Dual<N>> diff = pi - pj;
    const Dual<N> dist = dsqrt(dot(diff, diff));
    const Dual<N> sw = wi + wj;
    const Dual<N> w1 = wi / sw, w2 = wj / sw;
    const V3<Dual<N>> proj = scale(diff, dconst<N>(2.0f * r) / dist + (-1.0f));
    const V3<Dual<N>> dxi = scale(proj, w1);
    if (!counted || count <= 0) return dxi;
    const Dual<N> dxi2 = dot(dxi, dxi);
    const V3<Dual<N>> t1 = (dxi + pi - xi) - (scale(proj, -w2) + pj - xj);
    const V3<Dual<N>> nn = scale(diff, dconst<N>(1.0f) / dist);
    const V3<Dual<N>> tdx = t1 - scale(nn, dot(t1, nn));
    const Dual<N> tl2 = dot(tdx, tdx);
    V3<Dual<N>> f = scale(tdx, -w1);
    if (!(tl2.v <= C.fs * C.fs * dxi2.v)) f = scale(f, dmin(C.fd * dsqrt(dxi2 / tl2), 1.0f));
    return dxi + scale(f, 1.0f / (float)count);
}

// Pass A: c_k, from the same pairs and float operations as the forward.
__global__ void __launch_bounds__(kWalkThreads) k_adj_contact_count(SimConsts C, const float4 *__restrict__ P,
                                                                    const float *__restrict__ w,
                                                                    const int *__restrict__ off, int *__restrict__ count)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= C.n) return;
    const float4 pk4 = P[k];
    const float3 pk = f3(pk4);
    const int phk = phase_of(pk4);
    const float wk = w[k];
    int c = 0;
    auto test = [&](int j, float4 pj4) { return j != k && contact_pair(C, pk, phk, pj4); };
    auto body = [&](int j, float4 pj4) { c += contact_counted(C, pk, wk, f3(pj4), w[j]) ? 1 : 0; };
    walk_neighbors<true>(k, pk, 0, P, grid_view(C, scene_index(C, k), off), C, nullptr, -1, test, body);
    count[k] = c;
}

// Pass B: gIn = gOut + the pairs' Jacobians: those of k's own moves (its
// inputs as mover) and those of its neighbours' moves (its inputs as partner),
// gathered over the same pairs (the filter is symmetric).  Start-position and
// mass gradients add to gXs and gW.
__global__ void __launch_bounds__(kWalkThreads) k_adj_contact(SimConsts C, const float4 *__restrict__ P,
                                                              const float4 *__restrict__ Xs,
                                                              const float *__restrict__ w, const int *__restrict__ off,
                                                              const int *__restrict__ count,
                                                              const float4 *__restrict__ gOut,
                                                              float4 *__restrict__ gIn, float4 *__restrict__ gXs,
                                                              float *__restrict__ gW)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= C.n) return;
    const float4 pk4 = P[k];
    const float3 pk = f3(pk4), xk = ld3(Xs, k), gk = ld3(gOut, k);
    const int phk = phase_of(pk4);
    const float wk = w[k];
    const int ck = count[k];
    float acc[7] = {gk.x, gk.y, gk.z, 0.f, 0.f, 0.f, 0.f};  // p_k, X_k, w_k
    auto test = [&](int j, float4 pj4) { return j != k && contact_pair(C, pk, phk, pj4); };
    auto body = [&](int j, float4 pj4) {
        const float3 pj = f3(pj4), xj = ld3(Xs, j);
        const float wj = w[j];
        {  // k moves
            const V3<Dual<7>> out =
                dcontact<7>(C, dv3var<7>(pk, 0), dv3var<7>(xk, 3), dvar<7>(wk, 6), dv3<7>(pj), dv3<7>(xj),
                            dconst<7>(wj), contact_counted(C, pk, wk, pj, wj), ck);
#pragma unroll
            for (int q = 0; q < 7; ++q) acc[q] += vjp(out, gk, q);
        }
        {  // j moves, k is its partner
            const V3<Dual<7>> out =
                dcontact<7>(C, dv3<7>(pj), dv3<7>(xj), dconst<7>(wj), dv3var<7>(pk, 0), dv3var<7>(xk, 3),
                            dvar<7>(wk, 6), contact_counted(C, pj, wj, pk, wk), __ldg(count + j));
            const float3 gj = ld3(gOut, j);
#pragma unroll
            for (int q = 0; q < 7; ++q) acc[q] += vjp(out, gj, q);
        }
    };
    walk_neighbors<true>(k, pk, 0, P, grid_view(C, scene_index(C, k), off), C, nullptr, -1, test, body);
    gIn[k] = make_float4(acc[0], acc[1], acc[2], 0.f);
    gXs[k] = f4(add3(ld3(gXs, k), make_float3(acc[3], acc[4], acc[5])));
    gW[k] += acc[6];
}

// ---- dihedral bending (k_bending_terms, bp_constraints.cu) ----
// The four corrections of a quad as functions of its corners' positions and
// inverse scaled masses, on dual numbers (the same formulas as the forward).
template <int N>
__device__ __forceinline__ void dbending(const V3<Dual<N>> (&p)[4], const Dual<N> (&w)[4], float kb,
                                         V3<Dual<N>> (&out)[4])
{
#pragma unroll
    for (int c = 0; c < 4; ++c) out[c] = dv3<N>(make_float3(0.f, 0.f, 0.f));
    const V3<Dual<N>> e = p[1] - p[0], a = p[2] - p[0], b = p[3] - p[0];
    const V3<Dual<N>> ca = cross(e, a), cb = cross(e, b);
    const Dual<N> la = dsqrt(dot(ca, ca)), lb = dsqrt(dot(cb, cb));
    if (la.v <= 1e-5f || lb.v <= 1e-5f) return;
    const Dual<N> ila = dconst<N>(1.0f) / la, ilb = dconst<N>(1.0f) / lb;
    const V3<Dual<N>> n1 = scale(ca, ila), n2 = scale(cb, ilb);
    const Dual<N> d = dclamp(dot(n1, n2), -1.0f, 1.0f);
    const V3<Dual<N>> en1 = cross(e, n1), en2 = cross(e, n2);
    const V3<Dual<N>> an1 = cross(a, n1), an2 = cross(a, n2);
    const V3<Dual<N>> bn1 = cross(b, n1), bn2 = cross(b, n2);
    V3<Dual<N>> q[4];
    q[2] = scale(en2 - scale(en1, d), ila);
    q[3] = scale(en1 - scale(en2, d), ilb);
    q[1] = -scale(an2 - scale(an1, d), ila) - scale(bn1 - scale(bn2, d), ilb);
    q[0] = (-q[1] - q[2]) - q[3];
    Dual<N> den = w[0] * dot(q[0], q[0]);
#pragma unroll
    for (int c = 1; c < 4; ++c) den = den + w[c] * dot(q[c], q[c]);
    if (den.v <= 1e-5f) return;
    const Dual<N> num = dsqrt(dconst<N>(1.0f) - d * d) * (dacos(d) + (-3.141592f));
    const Dual<N> s = num / den;
#pragma unroll
    for (int c = 0; c < 4; ++c) out[c] = scale(q[c], (-w[c] * s) * kb);
}

// Per quad and corner c: the gradient of the loss through the quad's four
// corrections with respect to corner c's position (xyz) and inverse scaled
// mass (w), one dual evaluation per corner; laid out as the forward's terms.
__global__ void k_adj_bending_terms(int nq, const int4 *__restrict__ quads, const float4 *__restrict__ Pin,
                                    const float *__restrict__ w, const int *__restrict__ to_new, float kb,
                                    const float4 *__restrict__ gOut, float4 *__restrict__ terms)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int4 ids = quads[q];
    const int id[4] = {to_new[ids.x], to_new[ids.y], to_new[ids.z], to_new[ids.w]};
    float3 p[4], g[4];
    float wv[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        p[c] = ld3(Pin, id[c]);
        g[c] = ld3(gOut, id[c]);
        wv[c] = w[id[c]];
    }
#pragma unroll 1
    for (int ci = 0; ci < 4; ++ci) {
        V3<Dual<4>> P[4], D[4];
        Dual<4> W[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            P[c] = c == ci ? dv3var<4>(p[c], 0) : dv3<4>(p[c]);
            W[c] = c == ci ? dvar<4>(wv[c], 3) : dconst<4>(wv[c]);
        }
        dbending<4>(P, W, kb, D);
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[k] += vjp(D[c], g[c], k);
        terms[4 * (size_t)q + ci] = make_float4(acc[0], acc[1], acc[2], acc[3]);
    }
}

// gP += the terms of each particle's quads (CSR order), gW += their w parts.
__global__ void k_adj_bending_apply(int nn_, const int *__restrict__ node_ids, const int *__restrict__ ptr,
                                    const int *__restrict__ inc, const float4 *__restrict__ terms,
                                    const int *__restrict__ to_new, float4 *__restrict__ gP, float *__restrict__ gW)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn_) return;
    const int i = to_new[node_ids[t]];
    float3 g = ld3(gP, i);
    float gw = gW[i];
    for (int q = ptr[t]; q < ptr[t + 1]; ++q) {
        const float4 c = terms[inc[q]];
        g = add3(g, f3(c));
        gw += c.w;
    }
    gP[i] = f4(g);
    gW[i] = gw;
}

// ---- vorticity confinement and Akinci tension (k_post_a / k_post_b, bp_fluid.cu) ----
// Over the fluid neighbours j of the same phase within h (r_ij = p_i - p_j != 0),
// with G(r) the spiky gradient and H(r) its (even, symmetric) Jacobian:
//   pass A: w_i = sum_j (v_j - v_i) x G(r_ij);  n_i = h sum_j G(r_ij) / rho_j
//   pass B: eta_i = sum_j |w_j| G(r_ij);
//           v_i' = v_i + dt eps (eta_i / |eta_i|) x w_i   (where |eta_i|^2 > 1e-3)
//                + dt sum_j k_ij (F(|r_ij|) r_ij - gamma (n_i - n_j)),
//           k_ij = 2 rho0 / (rho_i + rho_j), F(r) = -gamma A(r) / r (A: Akinci's spline).
// Three gathers: eta-bar per particle; then pass B's adjoint (w-bar, n-bar,
// rho-bar, positions); then pass A's (velocities, positions, rho-bar).  Each
// sums a particle's terms as the mover and, through the symmetric pair set,
// its terms as the neighbour of its neighbours' sums.

// F(r) r and the product of its Jacobian F I + F' r r^T / |r| with u.
struct AkinciD {
    float F, Fp;
};
__device__ __forceinline__ AkinciD akinci_d(const SimConsts &C, float rl)
{
    const float t = (C.h - rl) * rl;
    const float two = rl >= C.half_h ? 1.0f : 2.0f;
    const float A = rl >= C.half_h ? C.c_akinci * t * t * t : 2.0f * C.c_akinci * t * t * t - C.c_akinci_off;
    const float Ap = two * C.c_akinci * 3.0f * t * t * (C.h - 2.0f * rl);
    AkinciD a;
    a.F = -C.tension * A / rl;
    a.Fp = -C.tension * (Ap / rl - A / (rl * rl));
    return a;
}
__device__ __forceinline__ float3 akinci_jac_mul(const AkinciD &a, float3 r, float rl, float3 u)
{
    return add3(mul3(u, a.F), mul3(r, a.Fp * dotf(r, u) / rl));
}
__device__ __forceinline__ float3 cross_f(float3 a, float3 b)
{
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// The pass-A neighbours of fluid particle k: body(j, p_j, r = p_k - p_j, |r|).
template <class B>
__device__ __forceinline__ void post_pairs(const SimConsts &C, int k, float3 pk, int phk, const float4 *__restrict__ P,
                                           const int *__restrict__ off, B &&body)
{
    auto test = [&](int j, float4 pj4) {
        const float3 r = sub3(pk, f3(pj4));
        const float d2 = dotf(r, r);
        return j != k && phase_of(pj4) == phk && d2 <= C.h2 && d2 > 0.f;
    };
    auto term = [&](int j, float4 pj4) {
        const float3 r = sub3(pk, f3(pj4));
        body(j, r, sqrtf(dotf(r, r)));
    };
    walk_neighbors<true>(k, pk, 0, P, grid_view(C, scene_index(C, k), off), C, nullptr, -1, test, term);
}

// eta-bar_i and the w-bar of i's own confinement term (zero where it is off).
__global__ void __launch_bounds__(kWalkThreads) k_adj_post_eta(SimConsts C, const float4 *__restrict__ P,
                                                               const int *__restrict__ off,
                                                               const float4 *__restrict__ Om,
                                                               const float4 *__restrict__ gVb,
                                                               float4 *__restrict__ etab, float4 *__restrict__ omb)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= C.n) return;
    const float4 pk4 = P[k];
    const int phk = phase_of(pk4);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    if (phk >= 0 || !C.use_vort) {
        etab[k] = zero;
        omb[k] = zero;
        return;
    }
    float3 eta = make_float3(0.f, 0.f, 0.f);
    post_pairs(C, k, f3(pk4), phk, P, off, [&](int j, float3 r, float rl) {
        eta = add3(eta, mul3(spiky_d(C, r, rl).g, Om[j].w));
    });
    const float e2 = dotf(eta, eta);
    if (!(e2 > 1e-3f)) {
        etab[k] = zero;
        omb[k] = zero;
        return;
    }
    const float el = sqrtf(e2);
    const float3 eh = mul3(eta, 1.0f / el), g = ld3(gVb, k), om = ld3(Om, k);
    const float a = C.dt * C.vort_eps;
    const float3 ehb = mul3(cross_f(om, g), a);  // (eta-hat x w) . g
    etab[k] = f4(mul3(sub3(ehb, mul3(eh, dotf(eh, ehb))), 1.0f / el));
    omb[k] = f4(mul3(cross_f(g, eh), a));
}

// Pass B's adjoint: w-bar (omb in, the full w-bar out in ombo), n-bar, and
// the density and position gradients (added to gRho and gX).
__global__ void __launch_bounds__(kWalkThreads) k_adj_post_b(SimConsts C, const float4 *__restrict__ P,
                                                             const int *__restrict__ off,
                                                             const float4 *__restrict__ Om,
                                                             const float4 *__restrict__ Nm,
                                                             const float4 *__restrict__ gVb,
                                                             const float4 *__restrict__ etab,
                                                             const float4 *__restrict__ omb,
                                                             float4 *__restrict__ ombo, float4 *__restrict__ nmb,
                                                             float *__restrict__ gRho, float4 *__restrict__ gX)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= C.n) return;
    const float4 pk4 = P[k];
    const int phk = phase_of(pk4);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    if (phk >= 0) {
        ombo[k] = zero;
        nmb[k] = zero;
        return;
    }
    const float rho0 = rest_density(C, scene_index(C, k));
    const float4 om4 = Om[k], nm4 = Nm[k];
    const float3 gk = ld3(gVb, k), ek = ld3(etab, k), nk = f3(nm4);
    const float rk = nm4.w, dt = C.dt, gam = C.tension;
    float abs_omb = 0.f, rb = 0.f;
    float3 pb = make_float3(0.f, 0.f, 0.f), nb = make_float3(0.f, 0.f, 0.f);
    post_pairs(C, k, f3(pk4), phk, P, off, [&](int j, float3 r, float rl) {
        const SpikyD sp = spiky_d(C, r, rl);
        const float4 omj = Om[j], nmj = Nm[j];
        if (C.use_vort) {
            const float3 ej = ld3(etab, j);
            pb = add3(pb, mul3(spiky_hess_mul(sp, r, rl, ek), omj.w));  // k's eta through r
            pb = sub3(pb, mul3(spiky_hess_mul(sp, r, rl, ej), om4.w));  // j's eta through r_jk = -r
            abs_omb -= dotf(ej, sp.g);                                   // j's eta: |w_k| G(-r)
        }
        if (C.use_akinci) {
            const AkinciD ak = akinci_d(C, rl);
            const float3 fco = mul3(r, ak.F);
            const float3 gj = ld3(gVb, j), nj = f3(nmj);
            const float sr = rk + nmj.w;
            const float kk = 2.0f * rho0 / sr, kd = -2.0f * rho0 / (sr * sr);
            // k moves: k_kj (fco(r) - gamma (n_k - n_j))
            nb = sub3(nb, mul3(gk, gam * dt * kk));
            rb += dt * kd * dotf(gk, sub3(fco, mul3(sub3(nk, nj), gam)));
            pb = add3(pb, mul3(akinci_jac_mul(ak, r, rl, gk), dt * kk));
            // j moves: k_jk (fco(-r) - gamma (n_j - n_k))
            nb = add3(nb, mul3(gj, gam * dt * kk));
            rb += dt * kd * dotf(gj, sub3(mul3(fco, -1.f), mul3(sub3(nj, nk), gam)));
            pb = sub3(pb, mul3(akinci_jac_mul(ak, r, rl, gj), dt * kk));
        }
    });
    float3 wb = ld3(omb, k);
    if (om4.w > 0.f) wb = add3(wb, mul3(f3(om4), abs_omb / om4.w));
    ombo[k] = f4(wb);
    nmb[k] = f4(nb);
    gRho[k] += rb;
    gX[k] = f4(add3(ld3(gX, k), pb));
}

// Pass A's adjoint: gV = gVb + the velocity terms of w; positions to gX,
// density to gRho.
__global__ void __launch_bounds__(kWalkThreads) k_adj_post_a(SimConsts C, const float4 *__restrict__ P,
                                                             const float4 *__restrict__ V, const int *__restrict__ off,
                                                             const float *__restrict__ rho,
                                                             const float4 *__restrict__ gVb,
                                                             const float4 *__restrict__ ombo,
                                                             const float4 *__restrict__ nmb,
                                                             float4 *__restrict__ gV, float *__restrict__ gRho,
                                                             float4 *__restrict__ gX)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= C.n) return;
    const float4 pk4 = P[k];
    const int phk = phase_of(pk4);
    float3 gv = ld3(gVb, k);
    if (phk >= 0) {
        gV[k] = f4(gv);
        return;
    }
    const float3 vk = ld3(V, k), wk = ld3(ombo, k), nk = ld3(nmb, k);
    const float rk = rho[k], h = C.h;
    float3 pb = make_float3(0.f, 0.f, 0.f);
    float rb = 0.f;
    post_pairs(C, k, f3(pk4), phk, P, off, [&](int j, float3 r, float rl) {
        const SpikyD sp = spiky_d(C, r, rl);
        const float3 vj = ld3(V, j);
        if (C.use_vort) {
            const float3 wj = ld3(ombo, j);
            // k's w: (v_j - v_k) x G(r)
            gv = sub3(gv, cross_f(sp.g, wk));
            pb = add3(pb, spiky_hess_mul(sp, r, rl, cross_f(wk, sub3(vj, vk))));
            // j's w: (v_k - v_j) x G(-r)
            gv = sub3(gv, cross_f(sp.g, wj));
            pb = sub3(pb, spiky_hess_mul(sp, r, rl, cross_f(wj, sub3(vk, vj))));
        }
        if (C.use_akinci) {
            const float3 nj = ld3(nmb, j);
            const float rj = rho[j];
            pb = add3(pb, mul3(spiky_hess_mul(sp, r, rl, nk), h / rj));  // k's n: G(r) / rho_j
            pb = sub3(pb, mul3(spiky_hess_mul(sp, r, rl, nj), h / rk));  // j's n: G(-r) / rho_k
            rb += h / (rk * rk) * dotf(nj, sp.g);
        }
    });
    gV[k] = f4(gv);
    gRho[k] += rb;
    gX[k] = f4(add3(ld3(gX, k), pb));
}

// ---- launchers ----

static int blocks(int n, int t = 256) { return (n + t - 1) / t; }

void adj_reorder(cudaStream_t st, const SimConsts &C, const int *order, const float4 *Xprev, const float4 *Vprev,
                 int stabilize, int inv_scaled, const float4 *gP, const float4 *gXs, const float4 *gVs,
                 const float *gW, float4 *gXprev, float4 *gVprev)
{
    if (C.n <= 0) return;
    k_adj_reorder<<<blocks(C.n), 256, 0, st>>>(C, order, Xprev, Vprev, stabilize, inv_scaled, gP, gXs, gVs, gW,
                                               gXprev, gVprev);
}
void adj_planes(cudaStream_t st, const SimConsts &C, const float4 *Xs, const float4 *Pin, float4 *gP, float4 *gXs)
{
    if (C.n <= 0) return;
    k_adj_planes<<<blocks(C.n), 256, 0, st>>>(C, Xs, Pin, gP, gXs);
}
void adj_commit(cudaStream_t st, int n, float inv_dt, const float4 *gX, const float4 *gV, float4 *gP, float4 *gXs,
                float4 *gVs, float *gW)
{
    if (n <= 0) return;
    k_adj_commit<<<blocks(n), 256, 0, st>>>(n, inv_dt, gX, gV, gP, gXs, gVs, gW);
}
void adj_immovable(cudaStream_t st, int k, const int *ids, const int *to_new, float4 *gP, float4 *gXs)
{
    if (k <= 0) return;
    k_adj_immovable<<<blocks(k), 256, 0, st>>>(k, ids, to_new, gP, gXs);
}
void adj_distance(cudaStream_t st, const DistanceArgs &a, const float4 *Pin, const float *w, const int *to_new,
                  float4 *gP, float *gW, float4 *G1, float4 *G2, float *g_stiff, float *g_rest)
{
    if (a.num_edges <= 0) return;
    k_adj_distance_edges<<<blocks(a.num_edges), 256, 0, st>>>(a.num_edges, a.pairs, a.params, Pin, w, to_new, gP, G1,
                                                              G2, g_stiff, g_rest);
    k_adj_distance_apply<<<blocks(a.num_nodes), 256, 0, st>>>(a.num_nodes, a.node_ids, a.node_ptr, a.node_inc, G1, G2,
                                                              to_new, gP, gW);
}
void adj_wind(cudaStream_t st, const SimConsts &C, const WindArgs &a, const float4 *Pin, const float4 *Vs,
              const float *mass, const int *to_new, float4 *gP, float4 *gVs, float4 *FG, float4 *FV, float4 *FW,
              float4 *g_wind)
{
    if (a.num_faces <= 0) return;
    k_adj_wind_faces<<<blocks(a.num_faces), 256, 0, st>>>(C, a.num_faces, a.faces, Pin, Vs, mass, to_new, gP, FG, FV,
                                                          FW);
    k_adj_wind_apply<<<blocks(a.num_nodes), 256, 0, st>>>(a.num_nodes, a.node_ids, a.node_ptr, a.node_inc, a.faces,
                                                          FG, FV, to_new, gP, gVs);
    k_adj_sum4<<<1, 1024, 0, st>>>(a.num_faces, FW, g_wind);
}
void adj_fluid(cudaStream_t st, const SimConsts &C, const float4 *Pin, const float *mass, const float *lam,
               const float *rho, const int *off, const float4 *gOut, const float *gRho, float *gLam, float4 *gPart,
               float4 *GD, float *rhob, float4 *gIn)
{
    if (C.n <= 0) return;
    const int b = blocks(C.n, kWalkThreads);
    k_adj_deltap<<<b, kWalkThreads, stage_bytes(C), st>>>(C, Pin, mass, lam, off, gOut, gLam, gPart);
    if (C.textbook) {
        k_adj_lambda_tb_prep<<<b, kWalkThreads, 0, st>>>(C, Pin, mass, off, gLam, gRho, GD, rhob);
        k_adj_lambda_tb<<<b, kWalkThreads, 0, st>>>(C, Pin, mass, off, GD, rhob, gPart, gOut, gIn);
    } else {
        k_adj_lambda<<<b, kWalkThreads, stage_bytes(C), st>>>(C, Pin, mass, rho, off, gLam, gPart, gOut, gRho, gIn);
    }
}
void adj_shape_matching(cudaStream_t st, const RigidArgs &a, const float4 *rot, const float4 *Pin, const int *to_new,
                        float4 *gP)
{
    if (a.num_bodies <= 0) return;
    k_adj_shape_matching<<<a.num_bodies, kAdjSmThreads, 0, st>>>(a, rot, Pin, to_new, gP);
}
void adj_xsph(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *V, const int *off,
              const float *mass, const float *rho, const float4 *gVout, float4 *gVin, float4 *gX, float *gRho)
{
    if (C.n <= 0) return;
    k_adj_xsph<<<blocks(C.n, kWalkThreads), kWalkThreads, stage_bytes(C), st>>>(C, P, V, off, mass, rho, gVout,
                                                                               gVin, gX, gRho);
}

void adj_contacts(cudaStream_t st, const SimConsts &C, const float4 *Pin, const float4 *Xs, const float *w,
                  const int *off, int *count, const float4 *gOut, float4 *gIn, float4 *gXs, float *gW)
{
    if (C.n <= 0) return;
    k_adj_contact_count<<<blocks(C.n, kWalkThreads), kWalkThreads, 0, st>>>(C, Pin, w, off, count);
    k_adj_contact<<<blocks(C.n, kWalkThreads), kWalkThreads, 0, st>>>(C, Pin, Xs, w, off, count, gOut, gIn, gXs, gW);
}

void adj_bending(cudaStream_t st, const BendingArgs &a, float kb, const float4 *Pin, const float *w, const int *to_new,
                 float4 *gP, float *gW)
{
    if (a.num_quads <= 0) return;
    k_adj_bending_terms<<<blocks(a.num_quads), 256, 0, st>>>(a.num_quads, a.quads, Pin, w, to_new, kb, gP, a.terms);
    k_adj_bending_apply<<<blocks(a.num_nodes), 256, 0, st>>>(a.num_nodes, a.node_ids, a.node_ptr, a.node_inc, a.terms,
                                                             to_new, gP, gW);
}

void adj_post(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *V, const float4 *Om,
              const float4 *Nm, const float *rho, const int *off, const float4 *gVb, float4 *gV, float4 *gX,
              float *gRho, float4 *etab, float4 *omb, float4 *ombo, float4 *nmb)
{
    if (C.n <= 0) return;
    const int b = blocks(C.n, kWalkThreads);
    k_adj_post_eta<<<b, kWalkThreads, 0, st>>>(C, P, off, Om, gVb, etab, omb);
    k_adj_post_b<<<b, kWalkThreads, 0, st>>>(C, P, off, Om, Nm, gVb, etab, omb, ombo, nmb, gRho, gX);
    k_adj_post_a<<<b, kWalkThreads, 0, st>>>(C, P, V, off, rho, gVb, ombo, nmb, gV, gRho, gX);
}

// ---- picking: the picked particle's position (and velocity) is overwritten
// with the target, so nothing before it reaches the loss through them ----

__global__ void k_adj_unpick(int id, const int *__restrict__ to_new, float4 *__restrict__ g1, float4 *__restrict__ g2)
{
    const int i = to_new[id];
    g1[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (g2) g2[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void k_adj_unpick_orig(int n, int id, const int *__restrict__ orig, float4 *__restrict__ g1,
                                  float4 *__restrict__ g2)
{
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < n; o += gridDim.x * blockDim.x)
        if (orig[o] == id) {
            g1[o] = make_float4(0.f, 0.f, 0.f, 0.f);
            g2[o] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
}

void adj_unpick(cudaStream_t st, int id, const int *to_new, float4 *g1, float4 *g2)
{
    k_adj_unpick<<<1, 1, 0, st>>>(id, to_new, g1, g2);
}

void adj_unpick_orig(cudaStream_t st, int n, int id, const int *orig, float4 *g1, float4 *g2)
{
    if (n <= 0) return;
    k_adj_unpick_orig<<<std::min(blocks(n), 1024), 256, 0, st>>>(n, id, orig, g1, g2);
}

}  // namespace bp
