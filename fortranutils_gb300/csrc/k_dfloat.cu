// k_dfloat.cu -- the mixed solver's outer iteration without FP64 arithmetic.
//
// GB300 issues FP64 at a small fraction of its FP32 rate, and the defect
// correction's level-1 work -- p += e and r = b - A p with the FP64
// coefficients, once per V-cycle -- was bound by the FP64 pipe.  Here p,
// the four coefficient arrays and b are held as double-float pairs (an FP32
// hi and an FP32 lo with hi + lo the value to about 48 significant bits)
// and both kernels run on the FP32 pipe, with the error-free transformations
// of Knuth (two-sum), Dekker (fast two-sum) and the FMA two-product:
//
//   two_sum(a, b)  = (s, e): s = fl(a + b), a + b = s + e exactly
//   fast_sum(a, b) = (s, e): the same when |a| >= |b|
//   two_prod(a, b) = (p, e): p = fl(a b), e = fma(a, b, -p), a b = p + e
//
// The residual of the double-float p is accurate to about 2^-47 of the
// largest term of A p, against 2^-53 in FP64; the solve's stopping test
// takes it, and the converged p is converted back to FP64 and confirmed by
// one FP64 residual (k_resid_outer), so the tolerance is met in FP64.
// Compiled without FMA contraction: every FMA below is written out.
#include <algorithm>

#include "k_common.cuh"
#include "kernels.h"

namespace {

__device__ __forceinline__ float2 two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return make_float2(s, e);
}

__device__ __forceinline__ float2 fast_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// a + b, both double-float (the accurate sum: lo parts added by two-sum too)
__device__ __forceinline__ float2 df_add(float2 a, float2 b)
{
    float2 s = two_sum(a.x, b.x);
    const float2 t = two_sum(a.y, b.y);
    s = fast_sum(s.x, __fadd_rn(s.y, t.x));
    return fast_sum(s.x, __fadd_rn(s.y, t.y));
}

// a + b, both double-float, with the lo parts added in FP32: the error is
// about 2^-24 of |a.lo + b.lo|, i.e. about 2^-48 of |a| + |b|, the order of
// the format itself; cheaper than df_add by nine operations
__device__ __forceinline__ float2 df_add_lo(float2 a, float2 b)
{
    const float2 s = two_sum(a.x, b.x);
    return fast_sum(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}

// a + b, b an FP32 value
__device__ __forceinline__ float2 df_add_f(float2 a, float b)
{
    const float2 s = two_sum(a.x, b);
    return fast_sum(s.x, __fadd_rn(s.y, a.y));
}

// a * b, both double-float (the lo * lo product is below the format)
__device__ __forceinline__ float2 df_mul(float2 a, float2 b)
{
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    return fast_sum(p, e);
}

__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ float2 split(double v)
{
    const float hi = __double2float_rn(v);
    return make_float2(hi, __double2float_rn(v - (double)hi));
}

__global__ void k_df_split(const double *__restrict__ src, float2 *__restrict__ dst, long n)
{
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        dst[q] = split(src[q]);
}

// b - shift (the block's interior mean of b, or 0) on the interior of level 1
__global__ void k_df_split_b(const BlkDev *__restrict__ blk, const double *__restrict__ b,
                             const double *__restrict__ shift, float2 *__restrict__ dst)
{
    const BlkDev bk = blk[blockIdx.y];
    const double s0 = shift ? shift[blockIdx.y] : 0.;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < bk.ncell; q += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        const long p = decode_interior(bk, q, i, j, k);
        dst[p] = split(b[p] - s0);
    }
}

// cycles (nullable, a device count): nothing to do when it is 0
__global__ void k_df_join(const float2 *__restrict__ src, double *__restrict__ dst, long n,
                          const double *__restrict__ cycles)
{
    if (cycles && *cycles == 0.) return;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const float2 v = src[q];
        dst[q] = (double)v.x + (double)v.y;
    }
}

// p += e on the interior of level 1, ghosts pushed as k_update does.
// Thread (x, y) of CTA (bx, by, bz): point i = 2 + 32 bx + x of row
// j = 2 + blockDim.y by + y of plane k = 2 + bz % maxnk of block
// bi0 + bz / maxnk.
template <typename Ix>
__global__ void k_df_update(const BlkDev *__restrict__ blk, float2 *__restrict__ p, const float *__restrict__ e,
                            const PushDev *__restrict__ push, int maxnk, int bi0)
{
    const int bz = (int)blockIdx.z / maxnk, k = (int)blockIdx.z - bz * maxnk + 2, bi = bi0 + bz;
    const int n0 = blk[bi].n[0], n1 = blk[bi].n[1], n2 = blk[bi].n[2];
    const int i = (int)(blockIdx.x * 32 + threadIdx.x) + 2, j = (int)(blockIdx.y * blockDim.y + threadIdx.y) + 2;
    if (k > n2 - 1 || j > n1 - 1 || i > n0 - 1) return;
    const Ix pp = (Ix)blk[bi].off3 + (i - 1) + (Ix)n0 * (j - 1) + (Ix)n0 * n1 * (k - 1);
    const float2 v = df_add_f(p[pp], e[pp]);
    p[pp] = v;
    if (push && (i == 2 || i == n0 - 1 || j == 2 || j == n1 - 1 || k == 2 || k == n2 - 1))
        push_ghosts(push + 6 * bi, blk[bi], i, j, k, v, p);
}

// r = b - A p in double-float (E, N, R, P as in k_resid_outer): r rounded
// to FP32 as the next cycle's right-hand side, per-CTA partial sums of r^2
// in FP64 (an FP32 square overflows above 1.8e19, which a diverging cycle
// reaches; summing in FP32 within [2^-60, 2^60] and in FP64 outside
// measured slower, 119 against 88 us on the mixing layer's level 1).
// A warp per (j, k) row of the block's interior, grid-stride over rows,
// lanes along i.
__global__ void __launch_bounds__(256) k_df_resid(const BlkDev *__restrict__ blk, const float2 *__restrict__ E,
                                                  const float2 *__restrict__ N, const float2 *__restrict__ R,
                                                  const float2 *__restrict__ P, const float2 *__restrict__ x,
                                                  const float2 *__restrict__ bb, float *__restrict__ rT,
                                                  double *__restrict__ partial)
{
    const BlkDev b = blk[blockIdx.y];
    const int ni = b.n[0] - 2;
    const unsigned nj = (unsigned)(b.n[1] - 2), nrow = nj * (unsigned)(b.n[2] - 2);
    const long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    const unsigned wpb = blockDim.x >> 5;
    double acc = 0.;
    for (unsigned row = blockIdx.x * wpb + (threadIdx.x >> 5); row < nrow; row += gridDim.x * wpb) {
        const unsigned k = row / nj;
        const long base = b.off3 + 1 + jo * (long)(row - k * nj + 1) + ko * (long)(k + 1);
        for (int iq = threadIdx.x & 31; iq < ni; iq += 32) {
            const long p = base + iq;
            float2 r = df_add_lo(bb[p], df_neg(df_mul(P[p], x[p])));
            r = df_add_lo(r, df_mul(E[p - 1], x[p - 1]));
            r = df_add_lo(r, df_mul(E[p], x[p + 1]));
            r = df_add_lo(r, df_mul(N[p - jo], x[p - jo]));
            r = df_add_lo(r, df_mul(N[p], x[p + jo]));
            r = df_add_lo(r, df_mul(R[p - ko], x[p - ko]));
            r = df_add_lo(r, df_mul(R[p], x[p + ko]));
            const float rf = __fadd_rn(r.x, r.y);
            rT[p] = rf;
            acc = __fma_rn((double)rf, (double)rf, acc);
        }
    }
    double v[1] = {acc};
    block_reduce_store<1>(v, partial + (blockIdx.y * (long)gridDim.x + blockIdx.x));
}

// out[0] = the sum of the partials (out[1], ||b||^2, is left as it is)
__global__ void k_df_sum_final(const double *__restrict__ partial, long nparts, double *__restrict__ out)
{
    double v[1] = {0.};
    for (long t = threadIdx.x; t < nparts; t += blockDim.x) v[0] += partial[t];
    __shared__ double r[1];
    block_reduce_store<1>(v, r);
    __syncthreads();
    if (threadIdx.x == 0) out[0] = r[0];
}

inline unsigned cap_grid(long n, int t, unsigned cap)
{
    const unsigned g = (unsigned)((n + t - 1) / t);
    return g > cap ? cap : (g ? g : 1);
}

} // namespace

namespace les {

void launch_df_split(const double *src, float2 *dst, long n, cudaStream_t st)
{
    k_df_split<<<cap_grid(n, 256, 4096), 256, 0, st>>>(src, dst, n);
    count_launch(1);
}

void launch_df_split_b(const BlkDev *blk, int nb, long maxcell, const double *b, const double *shift, float2 *dst,
                       cudaStream_t st)
{
    k_df_split_b<<<dim3(cap_grid(maxcell, 256, 2048), nb), 256, 0, st>>>(blk, b, shift, dst);
    count_launch(1);
}

void launch_df_join(const float2 *src, double *dst, long n, const double *cycles, cudaStream_t st)
{
    k_df_join<<<cap_grid(n, 256, 4096), 256, 0, st>>>(src, dst, n, cycles);
    count_launch(1);
}

void launch_df_update(const BlkDev *blk, int nb, const int maxn[3], float2 *p, const float *e, const PushDev *push,
                      bool wide, cudaStream_t st)
{
    const int maxnk = maxn[2] - 2, per = std::max(1, 65535 / maxnk);
    for (int bi0 = 0; bi0 < nb; bi0 += per) {
        const dim3 grid((unsigned)(maxn[0] + 29) / 32, (unsigned)(maxn[1] + 5) / 8,
                        (unsigned)(maxnk * std::min(per, nb - bi0)));
        if (wide)
            k_df_update<long><<<grid, dim3(32, 8), 0, st>>>(blk, p, e, push, maxnk, bi0);
        else
            k_df_update<int><<<grid, dim3(32, 8), 0, st>>>(blk, p, e, push, maxnk, bi0);
        count_launch(1);
    }
}

void launch_df_resid(const BlkDev *blk, int nb, long maxrow, const float2 *E, const float2 *N, const float2 *R,
                     const float2 *P, const float2 *x, const float2 *b, float *rT, double *partial, double *out,
                     cudaStream_t st)
{
    // a few CTAs per SM (so that the final sum reads few partials), every
    // warp the same number of rows
    const long cap = (1216 + nb - 1) / nb, per = (maxrow + 8 * cap - 1) / (8 * cap);
    const unsigned gx = (unsigned)std::max(1L, (maxrow + 8 * per - 1) / (8 * per));
    k_df_resid<<<dim3(gx, nb), 256, 0, st>>>(blk, E, N, R, P, x, b, rT, partial);
    k_df_sum_final<<<1, 256, 0, st>>>(partial, (long)gx * nb, out);
    count_launch(2);
}

} // namespace les
