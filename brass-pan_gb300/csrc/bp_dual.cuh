// bp_dual.cuh -- forward-mode dual numbers for the adjoint kernels.
//
// The adjoint of a small per-particle or per-constraint function (plane
// contacts, wind on one triangle, prediction and stabilisation) is the
// transpose of its Jacobian applied to the incoming gradient.  Evaluating the
// function once on Dual<N> inputs, seeded with the unit vectors of its N
// inputs, gives every column of the Jacobian at once.  The forward kernels
// keep their own bit-exact float code; these generic versions restate the
// same formulas for differentiation only.
#pragma once

#include <cuda_runtime.h>

namespace bp {

template <int N>
struct Dual {
    float v;
    float d[N];
};

template <int N>
__device__ __forceinline__ Dual<N> dconst(float v)
{
    Dual<N> r;
    r.v = v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = 0.f;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dvar(float v, int k)
{
    Dual<N> r = dconst<N>(v);
    r.d[k] = 1.f;
    return r;
}

#define BP_DUAL_BINOP(op, vexpr, dexpr)                                           \
    template <int N>                                                              \
    __device__ __forceinline__ Dual<N> operator op(const Dual<N> &a, const Dual<N> &b) \
    {                                                                             \
        Dual<N> r;                                                                \
        r.v = vexpr;                                                              \
        _Pragma("unroll") for (int k = 0; k < N; ++k) r.d[k] = dexpr;             \
        return r;                                                                 \
    }
BP_DUAL_BINOP(+, a.v + b.v, a.d[k] + b.d[k])
BP_DUAL_BINOP(-, a.v - b.v, a.d[k] - b.d[k])
BP_DUAL_BINOP(*, a.v * b.v, a.d[k] * b.v + a.v * b.d[k])
#undef BP_DUAL_BINOP

template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N> &a, const Dual<N> &b)
{
    Dual<N> r;
    const float inv = 1.0f / b.v;
    r.v = a.v * inv;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * inv;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N> &a, float s)
{
    Dual<N> r;
    r.v = a.v * s;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * s;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(float s, const Dual<N> &a) { return a * s; }
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N> &a, float s)
{
    Dual<N> r = a;
    r.v += s;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N> &a)
{
    Dual<N> r;
    r.v = -a.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dsqrt(const Dual<N> &a)
{
    Dual<N> r;
    r.v = sqrtf(a.v);
    const float g = r.v > 0.f ? 0.5f / r.v : 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * g;
    return r;
}
// min(a, s) as the forward's fminf picks it (a NaN picks s)
template <int N>
__device__ __forceinline__ Dual<N> dmin(const Dual<N> &a, float s)
{
    return (a.v < s) ? a : dconst<N>(s);
}
// min(max(a, lo), hi) as fminf(fmaxf(a, lo), hi) picks it
template <int N>
__device__ __forceinline__ Dual<N> dclamp(const Dual<N> &a, float lo, float hi)
{
    if (!(a.v > lo)) return dconst<N>(lo);
    if (!(a.v < hi)) return dconst<N>(hi);
    return a;
}
// arccos; d/da = -1 / sqrt(1 - a^2), taken as 0 where |a| = 1
template <int N>
__device__ __forceinline__ Dual<N> dacos(const Dual<N> &a)
{
    Dual<N> r;
    r.v = acosf(a.v);
    const float s = 1.0f - a.v * a.v;
    const float g = s > 0.f ? -1.0f / sqrtf(s) : 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * g;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dexp(const Dual<N> &a)
{
    Dual<N> r;
    r.v = expf(a.v);
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * r.v;
    return r;
}

// 3-vectors of any scalar type
template <class S>
struct V3 {
    S x, y, z;
};
template <class S>
__device__ __forceinline__ V3<S> operator+(const V3<S> &a, const V3<S> &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class S>
__device__ __forceinline__ V3<S> operator-(const V3<S> &a, const V3<S> &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class S>
__device__ __forceinline__ V3<S> operator-(const V3<S> &a) { return {-a.x, -a.y, -a.z}; }
template <class S, class T>
__device__ __forceinline__ V3<S> scale(const V3<S> &a, const T &s) { return {a.x * s, a.y * s, a.z * s}; }
template <class S>
__device__ __forceinline__ V3<S> scale_v(const S &s, float3 n) { return {s * n.x, s * n.y, s * n.z}; }
template <class S>
__device__ __forceinline__ S dot(const V3<S> &a, const V3<S> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class S>
__device__ __forceinline__ S dot(const V3<S> &a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class S>
__device__ __forceinline__ V3<S> cross(const V3<S> &a, const V3<S> &b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <int N>
__device__ __forceinline__ V3<Dual<N>> dv3(float3 a)
{
    return {dconst<N>(a.x), dconst<N>(a.y), dconst<N>(a.z)};
}
// a with its components seeded as inputs k0, k0 + 1, k0 + 2
template <int N>
__device__ __forceinline__ V3<Dual<N>> dv3var(float3 a, int k0)
{
    return {dvar<N>(a.x, k0), dvar<N>(a.y, k0 + 1), dvar<N>(a.z, k0 + 2)};
}
// sum over outputs of g . d(out)/d(input k)
template <int N>
__device__ __forceinline__ float vjp(const V3<Dual<N>> &out, float3 g, int k)
{
    return g.x * out.x.d[k] + g.y * out.y.d[k] + g.z * out.z.d[k];
}

}  // namespace bp
