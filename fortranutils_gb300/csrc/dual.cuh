// dual.cuh -- forward-mode dual numbers with N partial derivatives, for the
// local Jacobians of the adjoint and tangent-linear step (k_adjoint.cu).
// A Dual<N> carries a value and its derivatives with respect to N inputs;
// comparisons look at the value only, so branches follow the base state.
#pragma once
#include <cuda_runtime.h>

template <int N> struct Dual {
    double v;
    double d[N];
};

template <int N> __device__ __forceinline__ Dual<N> dconst(double a)
{
    Dual<N> r;
    r.v = a;
#pragma unroll
    for (int q = 0; q < N; q++) r.d[q] = 0.;
    return r;
}

__device__ __forceinline__ double val(double a) { return a; }
// a constant of the same number type as `like`
__device__ __forceinline__ double dconst_like(double, double a) { return a; }
template <int N> __device__ __forceinline__ Dual<N> dconst_like(const Dual<N> &, double a) { return dconst<N>(a); }
template <int N> __device__ __forceinline__ double val(const Dual<N> &a) { return a.v; }

#define DUAL_BIN(OP, VEXPR, DEXPR_DD, DEXPR_DS, DEXPR_SD)                                          \
    template <int N> __device__ __forceinline__ Dual<N> operator OP(const Dual<N> &a, const Dual<N> &b) \
    {                                                                                              \
        Dual<N> r;                                                                                 \
        r.v = VEXPR;                                                                               \
        _Pragma("unroll") for (int q = 0; q < N; q++) r.d[q] = DEXPR_DD;                          \
        return r;                                                                                  \
    }                                                                                              \
    template <int N> __device__ __forceinline__ Dual<N> operator OP(const Dual<N> &a, double bs)   \
    {                                                                                              \
        Dual<N> r;                                                                                 \
        const double b_v = bs;                                                                     \
        r.v = a.v OP b_v;                                                                          \
        _Pragma("unroll") for (int q = 0; q < N; q++) r.d[q] = DEXPR_DS;                          \
        return r;                                                                                  \
    }                                                                                              \
    template <int N> __device__ __forceinline__ Dual<N> operator OP(double as, const Dual<N> &b)   \
    {                                                                                              \
        Dual<N> r;                                                                                 \
        const double a_v = as;                                                                     \
        r.v = a_v OP b.v;                                                                          \
        _Pragma("unroll") for (int q = 0; q < N; q++) r.d[q] = DEXPR_SD;                          \
        return r;                                                                                  \
    }

DUAL_BIN(+, a.v + b.v, a.d[q] + b.d[q], a.d[q], b.d[q])
DUAL_BIN(-, a.v - b.v, a.d[q] - b.d[q], a.d[q], -b.d[q])
DUAL_BIN(*, a.v * b.v, a.d[q] * b.v + a.v * b.d[q], a.d[q] * b_v, a_v * b.d[q])
DUAL_BIN(/, a.v / b.v, (a.d[q] * b.v - a.v * b.d[q]) / (b.v * b.v), a.d[q] / b_v,
         -a_v * b.d[q] / (b.v * b.v))
#undef DUAL_BIN

template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N> &a)
{
    Dual<N> r;
    r.v = -a.v;
#pragma unroll
    for (int q = 0; q < N; q++) r.d[q] = -a.d[q];
    return r;
}

template <int N> __device__ __forceinline__ Dual<N> sqrt(const Dual<N> &a)
{
    Dual<N> r;
    r.v = ::sqrt(a.v);
    const double h = 0.5 / r.v;
#pragma unroll
    for (int q = 0; q < N; q++) r.d[q] = a.d[q] * h;
    return r;
}

template <int N> __device__ __forceinline__ Dual<N> log(const Dual<N> &a)
{
    Dual<N> r;
    r.v = ::log(a.v);
#pragma unroll
    for (int q = 0; q < N; q++) r.d[q] = a.d[q] / a.v;
    return r;
}

template <int N> __device__ __forceinline__ Dual<N> fabs(const Dual<N> &a) { return a.v < 0. ? -a : a; }

#define DUAL_CMP(OP)                                                                               \
    template <int N> __device__ __forceinline__ bool operator OP(const Dual<N> &a, double b) { return a.v OP b; } \
    template <int N> __device__ __forceinline__ bool operator OP(const Dual<N> &a, const Dual<N> &b) { return a.v OP b.v; }
DUAL_CMP(<)
DUAL_CMP(>)
DUAL_CMP(<=)
DUAL_CMP(>=)
#undef DUAL_CMP
