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
    pdl_wait();
    pdl_trigger();
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        dst[q] = split(src[q]);
}

// b - shift (the block's interior mean of b, or 0) on the interior of level 1
__global__ void k_df_split_b(const BlkDev *__restrict__ blk, const double *__restrict__ b,
                             const double *__restrict__ shift, float2 *__restrict__ dst)
{
    pdl_wait();
    pdl_trigger();
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
    pdl_wait();
    pdl_trigger();
    if (cycles && *cycles == 0.) return;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const float2 v = src[q];
        dst[q] = (double)v.x + (double)v.y;
    }
}

// p += e on the interior of level 1, ghosts pushed as k_update does.
// Thread (x, y) of CTA (bx, by, bz): point i = 2 + 32 bx + x of row
// j = 2 + blockDim.y by + y of the (block, plane) zmap[z0 + bz].
template <typename Ix>
__global__ void k_df_update(const BlkDev *__restrict__ blk, float2 *__restrict__ p, const float *__restrict__ e,
                            const PushDev *__restrict__ push, const int2 *__restrict__ zmap, int z0)
{
    const int2 bk = zmap[z0 + blockIdx.z];
    const int bi = bk.x, k = bk.y;
    const int n0 = blk[bi].n[0], n1 = blk[bi].n[1], n2 = blk[bi].n[2];
    const int i = (int)(blockIdx.x * 32 + threadIdx.x) + 2, j = (int)(blockIdx.y * blockDim.y + threadIdx.y) + 2;
    if (k > n2 - 1 || j > n1 - 1 || i > n0 - 1) return;
    const Ix pp = (Ix)blk[bi].off3 + (i - 1) + (Ix)n0 * (j - 1) + (Ix)n0 * n1 * (k - 1);
    pdl_wait();
    pdl_trigger();
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
    pdl_wait();
    pdl_trigger();
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

// Separable double-float factors of the level-1 FP64 couplings, the
// factorisation the FP32 solver's tables use (k_mf_extract): E(i, j, k) =
// E2(i, j) Ez(k) with E2 the couplings of plane kr and Ez(k) their ratio
// along the reference column (i0, j0); the same for N and R.  The factors
// are formed in FP64 and stored as double-float pairs.  bit 16: a zero
// coupling on the reference column.
__global__ void k_df_mf_extract(const BlkDev *__restrict__ blk, const double *__restrict__ E,
                                const double *__restrict__ N, const double *__restrict__ R, DfTab t,
                                int *__restrict__ bad)
{
    const BlkDev b = blk[blockIdx.y];
    const int n0 = b.n[0], n1 = b.n[1], n2 = b.n[2];
    const long jo = n0, ko = (long)n0 * n1;
    const int i0 = (n0 + 1) / 2, j0 = (n1 + 1) / 2, kr = (n2 + 1) / 2;
    const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q < (long)n0 * n1) {
        const long p = b.off3 + q + ko * (kr - 1);
        t.E2[b.off2 + q] = split(E[p]);
        t.N2[b.off2 + q] = split(N[p]);
        t.R2[b.off2 + q] = split(R[p]);
    }
    if (q < n2) {
        const long pc = b.off3 + (i0 - 1) + jo * (j0 - 1);
        const double e0 = E[pc + ko * (kr - 1)], nn0 = N[pc + ko * (kr - 1)], r0 = R[pc + ko * (kr - 1)];
        if (e0 == 0. || nn0 == 0. || r0 == 0.) {
            atomicOr(bad, 16);
            return;
        }
        t.Ez[b.off1k + q] = split(E[pc + ko * q] / e0);
        t.Nz[b.off1k + q] = split(N[pc + ko * q] / nn0);
        t.Rz[b.off1k + q] = split(R[pc + ko * q] / r0);
    }
}

__device__ __forceinline__ double df_val(float2 a) { return (double)a.x + (double)a.y; }

// Every interior point's six couplings from the factors within tol * ap of
// the FP64 arrays (else bit 1), and ap within tol * ap of their sum (else
// bit 2: the diagonal is then read from its array)
__global__ void k_df_mf_check(const BlkDev *__restrict__ blk, const double *__restrict__ E,
                              const double *__restrict__ N, const double *__restrict__ R,
                              const double *__restrict__ P, DfTab t, double tol, int *__restrict__ bad)
{
    const BlkDev b = blk[blockIdx.y];
    const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    const long p = decode_interior(b, q, i, j, k);
    const long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    const long ij = b.off2 + (i - 1) + jo * (j - 1), kk = b.off1k + (k - 1);
    const double ez = df_val(t.Ez[kk]), nz = df_val(t.Nz[kk]), r2 = df_val(t.R2[ij]);
    const double m[6] = {df_val(t.E2[ij - 1]) * ez, df_val(t.E2[ij]) * ez, df_val(t.N2[ij - jo]) * nz,
                         df_val(t.N2[ij]) * nz,     r2 * df_val(t.Rz[kk - 1]), r2 * df_val(t.Rz[kk])};
    const double ref[6] = {E[p - 1], E[p], N[p - jo], N[p], R[p - ko], R[p]};
    const double ap = fabs(P[p]);
    int f = 0;
    for (int c = 0; c < 6; c++)
        if (!(fabs(m[c] - ref[c]) <= tol * ap)) f |= 1;
    const double sum = ((m[0] + m[1]) + (m[2] + m[3])) + (m[4] + m[5]);
    if (!(fabs(sum - P[p]) <= tol * ap)) f |= 2;
    if (f) atomicOr(bad, f);
}

// k_df_resid with the couplings from the separable factors (df_mul of a
// 2-D and a 1-D pair) and, where P is NULL, the diagonal as their sum:
// the residual reads x, b and writes rT only (20 of k_df_resid's 52 B per
// point); the factors stay in L2.
__global__ void __launch_bounds__(256) k_df_resid_mf(const BlkDev *__restrict__ blk, DfTab t,
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
    pdl_wait();
    pdl_trigger();
    for (unsigned row = blockIdx.x * wpb + (threadIdx.x >> 5); row < nrow; row += gridDim.x * wpb) {
        const unsigned k = row / nj, jr = row - k * nj;
        const long base = b.off3 + 1 + jo * (long)(jr + 1) + ko * (long)(k + 1);
        const long ijb = b.off2 + 1 + jo * (long)(jr + 1), kk = b.off1k + k + 1;
        const float2 ez = t.Ez[kk], nz = t.Nz[kk], rzl = t.Rz[kk - 1], rzr = t.Rz[kk];
        for (int iq = threadIdx.x & 31; iq < ni; iq += 32) {
            const long p = base + iq, ij = ijb + iq;
            const float2 r2 = t.R2[ij];
            const float2 cw = df_mul(t.E2[ij - 1], ez), ce = df_mul(t.E2[ij], ez);
            const float2 cs = df_mul(t.N2[ij - jo], nz), cn = df_mul(t.N2[ij], nz);
            const float2 cl = df_mul(r2, rzl), cr = df_mul(r2, rzr);
            // the couplings are positive: their sum has no cancellation, and
            // the lo parts added in FP32 keep it to about 2^-48
            const float2 ap =
                P ? P[p] : df_add_lo(df_add_lo(df_add_lo(cw, ce), df_add_lo(cs, cn)), df_add_lo(cl, cr));
            float2 r = df_add_lo(bb[p], df_neg(df_mul(ap, x[p])));
            r = df_add_lo(r, df_mul(cw, x[p - 1]));
            r = df_add_lo(r, df_mul(ce, x[p + 1]));
            r = df_add_lo(r, df_mul(cs, x[p - jo]));
            r = df_add_lo(r, df_mul(cn, x[p + jo]));
            r = df_add_lo(r, df_mul(cl, x[p - ko]));
            r = df_add_lo(r, df_mul(cr, x[p + ko]));
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
    pdl_wait();
    pdl_trigger();
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
    launch_pdl(k_df_split, dim3(cap_grid(n, 256, 4096)), dim3(256), 0, st, src, dst, n);
    count_launch(1);
}

void launch_df_split_b(const BlkDev *blk, int nb, long maxcell, const double *b, const double *shift, float2 *dst,
                       cudaStream_t st)
{
    launch_pdl(k_df_split_b, dim3(cap_grid(maxcell, 256, 2048), nb), dim3(256), 0, st, blk, b, shift, dst);
    count_launch(1);
}

void launch_df_join(const float2 *src, double *dst, long n, const double *cycles, cudaStream_t st)
{
    launch_pdl(k_df_join, dim3(cap_grid(n, 256, 4096)), dim3(256), 0, st, src, dst, n, cycles);
    count_launch(1);
}

void launch_df_update(const BlkDev *blk, int nb, const int maxn[3], float2 *p, const float *e, const PushDev *push,
                      bool wide, ZMap zm, cudaStream_t st)
{
    (void)nb;
    for (int z0 = 0; z0 < zm.n; z0 += 65535) {
        const dim3 grid((unsigned)(maxn[0] + 29) / 32, (unsigned)(maxn[1] + 5) / 8, (unsigned)std::min(65535, zm.n - z0));
        if (wide)
            launch_pdl(k_df_update<long>, grid, dim3(32, 8), 0, st, blk, p, e, push, zm.map, z0);
        else
            launch_pdl(k_df_update<int>, grid, dim3(32, 8), 0, st, blk, p, e, push, zm.map, z0);
        count_launch(1);
    }
}

int launch_df_mf(const BlkDev *blk, int nb, long maxcell, long max2d, int maxn2, const double *E, const double *N,
                 const double *R, const double *P, const DfTab &t, double tol, int *bad, cudaStream_t st)
{
    const long m = std::max(max2d, (long)maxn2);
    k_df_mf_extract<<<dim3((unsigned)((m + 255) / 256), nb), 256, 0, st>>>(blk, E, N, R, t, bad);
    k_df_mf_check<<<dim3((unsigned)((maxcell + 255) / 256), nb), 256, 0, st>>>(blk, E, N, R, P, t, tol, bad);
    count_launch(2);
    return 0;
}

void launch_df_resid_mf(const BlkDev *blk, int nb, long maxrow, const DfTab &t, const float2 *P, const float2 *x,
                        const float2 *b, float *rT, double *partial, double *out, cudaStream_t st)
{
    const long cap = (1216 + nb - 1) / nb, per = (maxrow + 8 * cap - 1) / (8 * cap);
    const unsigned gx = (unsigned)std::max(1L, (maxrow + 8 * per - 1) / (8 * per));
    launch_pdl(k_df_resid_mf, dim3(gx, nb), dim3(256), 0, st, blk, t, P, x, b, rT, partial);
    launch_pdl(k_df_sum_final, dim3(1), dim3(256), 0, st, (const double *)partial, (long)gx * nb, out);
    count_launch(2);
}

void launch_df_resid(const BlkDev *blk, int nb, long maxrow, const float2 *E, const float2 *N, const float2 *R,
                     const float2 *P, const float2 *x, const float2 *b, float *rT, double *partial, double *out,
                     cudaStream_t st)
{
    // a few CTAs per SM (so that the final sum reads few partials), every
    // warp the same number of rows
    const long cap = (1216 + nb - 1) / nb, per = (maxrow + 8 * cap - 1) / (8 * cap);
    const unsigned gx = (unsigned)std::max(1L, (maxrow + 8 * per - 1) / (8 * per));
    launch_pdl(k_df_resid, dim3(gx, nb), dim3(256), 0, st, blk, E, N, R, P, x, b, rT, partial);
    launch_pdl(k_df_sum_final, dim3(1), dim3(256), 0, st, (const double *)partial, (long)gx * nb, out);
    count_launch(2);
}

} // namespace les
