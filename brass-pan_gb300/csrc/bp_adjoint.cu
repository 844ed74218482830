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
// collision), wind, reference-mode fluid density / lambda / position
// correction (with s_corr and the per-pair clamp), distance constraints,
// shape matching (rotation differentiated at its fixed point), immovables,
// the velocity update and reference-mode XSPH.
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

// The pairs of particle k that pass test, in walk order: term(j, P[j]).
// With C.nbr the walk records the pairs that pass `record` (a superset of
// test's) and the terms of those that pass test are summed over the list
// (four gathers at a time); the list's count goes to C.nbr_count[k] (-1:
// overflow), so that a later pass over the same positions can read it.
// Without lists, or past the list's capacity, the terms run inside the walk.
template <class R, class T, class B>
__device__ __forceinline__ void record_then_sum(const SimConsts &C, int k, float3 pk, const float4 *__restrict__ P,
                                                const GridView &v, const StageShared *S, int g, R &record, T &test,
                                                B &term)
{
    int cnt = -1;
    if (C.nbr) {
        ListWriter list(C.nbr, C.nbr_cap, C.n, k);
        walk_neighbors<true>(k, pk, 0, P, v, C, S, g, record, [&](int j, float4) { list.push(j); });
        cnt = list.finish();
        if (C.nbr_count) C.nbr_count[k] = cnt;
        if (cnt >= 0)
            for_each_in_list<false>(C.nbr, C.n, k, cnt, P, [&](int j, float4 pj) {
                if (test(j, pj)) term(j, pj);
            });
    }
    if (cnt < 0) walk_neighbors<true>(k, pk, 0, P, v, C, S, g, test, term);
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
    auto test = [&](int j, float4 pj4) {
        const float3 r = sub3(pk, f3(pj4));
        const float d2 = dotf(r, r);
        const bool inc = (j > k) ? (phk < 0) : (phase_of(pj4) < 0);
        return j != k && d2 <= C.h2 && d2 > 0.f && inc;
    };
    auto term = [&](int j, float4 pj4) {
            const float3 r = sub3(pk, f3(pj4));
            const float d2 = dotf(r, r);
            const float rl = sqrtf(d2);
            const SpikyD sp = spiky_d(C, r, rl);
            float s = lk + lam[j];
            float3 dsc = make_float3(0.f, 0.f, 0.f);  // d scorr / d r
            if (C.scorr_on) {
                const float x = poly6(C, d2) * C.scorr_inv_wq;
                s -= C.scorr_k * ipowf(x, C.scorr_ni);
                if (C.scorr_ni > 0)
                    dsc = mul3(poly6_grad(C, r, d2), C.scorr_k * C.scorr_ni * ipowf(x, C.scorr_ni - 1) * C.scorr_inv_wq);
            }
            // term of dp_k: (m_j / rho0) clamp(s gradW(r))
            const float3 u1b = mul3(clamp_vjp(C, mul3(sp.g, s), gk), mass[j] * inv_rho0);
            const float sb1 = dotf(u1b, sp.g);
            const float3 rb1 = sub3(mul3(spiky_hess_mul(sp, r, rl, u1b), s), mul3(dsc, sb1));
            // term of dp_j: (m_k / rho0) clamp(s gradW(-r))
            const float3 g_neg = mul3(sp.g, -1.f);
            const float3 u2b = mul3(clamp_vjp(C, mul3(g_neg, s), ld3(gOut, j)), mk * inv_rho0);
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
    record_then_sum(C, k, pk, P, grid_view(C, sc, off), &S, g, within, test, term);
    gLam[k] = lb;
    gPart[k] = f4(pb);
}

// Pass B: the density gradient; gP (in) = gOut + gPart + density terms.  It
// sums over the list pass A recorded at the same positions (every j != k
// within h, in walk order) and walks only where that list overflowed.
__global__ void __launch_bounds__(kWalkThreads) k_adj_lambda(SimConsts C, const float4 *__restrict__ P,
                                                             const float *__restrict__ mass,
                                                             const float *__restrict__ rho, const int *__restrict__ off,
                                                             const float *__restrict__ gLam,
                                                             const float4 *__restrict__ gPart,
                                                             const float4 *__restrict__ gOut, float4 *__restrict__ gIn)
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
        if (C.clamp_c && !(rho[j] / rho0 - 1.0f > 0.f)) return 0.f;
        return -gLam[j] / (C.lambda_den * rho0);
    };
    const float rbk = rho_bar(k, phk);
    const float mk = mass[k] * (phk < 0 ? 1.f : C.solid_scale);
    float3 pb = make_float3(0.f, 0.f, 0.f);
    auto test = [&](int j, float4 pj4) { return j != k && dotf(sub3(pk, f3(pj4)), sub3(pk, f3(pj4))) <= C.h2; };
    auto term = [&](int j, float4 pj4) {
        const int phj = phase_of(pj4);
        const float3 r = sub3(pk, f3(pj4));
        const float3 gw = poly6_grad(C, r, dotf(r, r));
        if (j > k) pb = add3(pb, mul3(gw, rbk * mass[j] * (phj < 0 ? 1.f : C.solid_scale)));
        else pb = add3(pb, mul3(gw, rho_bar(j, phj) * mk));
    };
    const int cnt = (C.nbr && C.nbr_count) ? __ldg(C.nbr_count + k) : -1;
    if (cnt >= 0) for_each_in_list(C.nbr, C.n, k, cnt, P, term);  // pass A's list: exactly test's pairs
    else walk_neighbors<true>(k, pk, 0, P, grid_view(C, sc, off), C, &S, g, test, term);
    gIn[k] = f4(add3(add3(ld3(gOut, k), ld3(gPart, k)), pb));
}

// ---- XSPH, reference mode: v'_i = v_i + c sum_j W6(r_ij) (v_j - v_i) ----
// Positions are the committed ones; gX receives their gradient.

__global__ void __launch_bounds__(kWalkThreads) k_adj_xsph(SimConsts C, const float4 *__restrict__ P,
                                                           const float4 *__restrict__ V, const int *__restrict__ off,
                                                           const float4 *__restrict__ gVout, float4 *__restrict__ gVin,
                                                           float4 *__restrict__ gX)
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
    float3 gv = go, gp = make_float3(0.f, 0.f, 0.f);
    auto test = [&](int j, float4 pj4) {
        const float3 r = sub3(pi, f3(pj4));
        return j != i && phase_of(pj4) == phi && dotf(r, r) <= C.h2;
    };
    auto term = [&](int j, float4 pj4) {
        const float3 r = sub3(pi, f3(pj4));
        const float d2 = dotf(r, r);
        const float w = poly6(C, d2);
        const float3 gj = ld3(gVout, j);
        gv = add3(gv, mul3(sub3(gj, go), C.xsph_c * w));
        const float3 dv = sub3(ld3(V, j), vi);
        gp = add3(gp, mul3(poly6_grad(C, r, d2), C.xsph_c * dotf(dv, sub3(go, gj))));
    };
    record_then_sum(C, i, pi, P, grid_view(C, scene_index(C, i), off), &S, g, test, test, term);
    gVin[i] = f4(gv);
    gX[i] = f4(add3(ld3(gX, i), gp));
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
               const float *rho, const int *off, const float4 *gOut, float *gLam, float4 *gPart, float4 *gIn)
{
    if (C.n <= 0) return;
    k_adj_deltap<<<blocks(C.n, kWalkThreads), kWalkThreads, stage_bytes(C), st>>>(C, Pin, mass, lam, off, gOut, gLam, gPart);
    k_adj_lambda<<<blocks(C.n, kWalkThreads), kWalkThreads, stage_bytes(C), st>>>(C, Pin, mass, rho, off, gLam, gPart, gOut, gIn);
}
void adj_shape_matching(cudaStream_t st, const RigidArgs &a, const float4 *rot, const float4 *Pin, const int *to_new,
                        float4 *gP)
{
    if (a.num_bodies <= 0) return;
    k_adj_shape_matching<<<a.num_bodies, kAdjSmThreads, 0, st>>>(a, rot, Pin, to_new, gP);
}
void adj_xsph(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *V, const int *off,
              const float4 *gVout, float4 *gVin, float4 *gX)
{
    if (C.n <= 0) return;
    k_adj_xsph<<<blocks(C.n, kWalkThreads), kWalkThreads, stage_bytes(C), st>>>(C, P, V, off, gVout, gVin, gX);
}

}  // namespace bp
