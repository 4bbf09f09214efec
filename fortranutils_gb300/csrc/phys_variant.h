// phys_variant.h -- the two builds of the FP64 physics units.
//
// k_phys.cu and k_sgs.cu are compiled twice.  The exact build (namespace
// les_exact, -fmad=false) keeps the reference's operation order, so every
// product, sum and quotient rounds as the Fortran FP64 does.  The fast build
// (namespace les_fast, -DLES_FAST_PHYS, FMA contraction on) multiplies by
// reciprocal metric tables instead of dividing by the metrics, takes the
// WALE powers 1.5, 2.5 and 1.25 through sqrt and the filter width from
// separable tables: each of those changes a result by a few units in the
// last place, not more, and GB300 issues FP64 slowly enough that the
// divisions and powers are most of these kernels' time.
#pragma once

#if defined(LES_F32_PHYS)
// the FP32-arithmetic build (gen_f32.py): FP64 fields read through LdF
#define LES_PHYS_NS les_f32
#define QDIV(x, d, rd) ((x) * (rd))
typedef float real;
// Read-only views for the FP32 build.  LdF: an FP64 field, converted on
// load.  LdM: a metric table, which the host passes as an FP32 copy with
// bit 0 of the pointer set (the conversion of an FP64 load runs on the
// FP64 pipe).  Each view masks its pointer once, to the alignment of its
// element type, so a pointer of the other kind can only read wrong values
// (which the parity tests would show), never from a misaligned address.
// Neither converts back to a raw pointer.
struct LdF {
    const double *p;
    __host__ __device__ __forceinline__ LdF(const double *q) : p((const double *)((unsigned long long)q & ~7ull)) {}
    __device__ __forceinline__ float operator[](long i) const { return (float)p[i]; }
    __device__ __forceinline__ LdF operator+(long o) const { return LdF(p + o); }
    __device__ __forceinline__ LdF operator-(long o) const { return LdF(p - o); }
};
struct LdM {
    const float *p;
    __host__ __device__ __forceinline__ LdM(const double *q) : p((const float *)((unsigned long long)q & ~3ull)) {}
    __host__ __device__ __forceinline__ LdM(const float *q) : p(q) {}
    __device__ __forceinline__ float operator[](long i) const { return p[i]; }
    __device__ __forceinline__ LdM operator+(long o) const { return LdM(p + o); }
    __device__ __forceinline__ LdM operator-(long o) const { return LdM(p - o); }
};
// an L2 load (__ldcg) through a field view (the scalar sweep's in-place field)
__device__ __forceinline__ float ldcg_f(LdF v) { return (float)__ldcg(v.p); }
#elif defined(LES_FAST_PHYS)
#define LES_PHYS_NS les_fast
// x / d, with rd = 1 / d precomputed
#define QDIV(x, d, rd) ((x) * (rd))
#else
#define LES_PHYS_NS les_exact
#define QDIV(x, d, rd) ((x) / (d))
#endif
