// k_fast.cu -- kernels of the fast pressure solvers (LES_PSOLVE_FP64 and
// LES_PSOLVE_MIXED).  Compiled with FMA contraction on.
//
// The operator is the reference's 7-point finite-volume matrix (coeff_p,
// code/coeff_p_block.F) stored in a compressed form per multigrid level:
//   E[p] couples p and p+1, N[p] couples p and p+jo, R[p] couples p and
//   p+ko, D[p] = 1/ap[p].
// Because coeff_p sets aw(i) = ae(i-1), as(j) = an(j-1), al(k) = ar(k-1),
// the west coefficient of p is E[p-1]; the ghost slots E[i=1], N[j=1],
// R[k=1] hold aw, as, al of the first interior point (non-zero only on
// periodic / interface sides).  k_conv_coef checks that pairing and refuses
// coefficients that lack it.
//
// The V-cycle is the reference's (code/lmg_solve.F) with the lexicographic
// SOR smoother replaced by red-black SOR, the restriction fused with the
// residual (8-child sum, code/rest_block.F:138-141) and the trilinear
// prolongation of code/prol_block.F, whose "coarse ghost := interior
// neighbour" rule (prol_block.F:325-357) is applied by clamping the coarse
// index instead of writing the ghosts.
#include "k_common.cuh"
#include "kernels.h"

template <typename T> struct Lvl {
    T *E, *N, *R, *D;
};

// ---- coefficient conversion (once per coefficient set) --------------------
template <typename T>
__global__ void k_conv_coef(const BlkDev *__restrict__ blk, const double *__restrict__ ap,
                            const double *__restrict__ aw, const double *__restrict__ ae,
                            const double *__restrict__ as, const double *__restrict__ an,
                            const double *__restrict__ al, const double *__restrict__ ar, T *E,
                            T *N, T *R, T *D, double *E64, double *N64, double *R64,
                            double *P64, int *bad)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long p = decode_interior(b, q, i, j, k);
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    E[p] = (T)ae[p];
    N[p] = (T)an[p];
    R[p] = (T)ar[p];
    D[p] = (T)(1.0 / ap[p]);
    if (i == 2) E[p - 1] = (T)aw[p];
    else if (aw[p] != ae[p - 1]) atomicOr(bad, 1);
    if (j == 2) N[p - jo] = (T)as[p];
    else if (as[p] != an[p - jo]) atomicOr(bad, 2);
    if (k == 2) R[p - ko] = (T)al[p];
    else if (al[p] != ar[p - ko]) atomicOr(bad, 4);
    // a row whose diagonal exceeds its off-diagonal sum makes the operator
    // non-singular (bit 8); coeff_p's pure-Neumann/periodic rows never do
    double off = aw[p] + ae[p] + as[p] + an[p] + al[p] + ar[p];
    if (fabs(ap[p] - off) > 1e-12 * fabs(ap[p])) atomicOr(bad, 8);
    if (E64) {
        E64[p] = ae[p];
        N64[p] = an[p];
        R64[p] = ar[p];
        P64[p] = ap[p];
        if (i == 2) E64[p - 1] = aw[p];
        if (j == 2) N64[p - jo] = as[p];
        if (k == 2) R64[p - ko] = al[p];
    }
}

// ---- tables of the fast physics kernels -------------------------------------
struct RecipJob {
    const double *src[24];
    double *dst[24];
};

__global__ void k_recip(RecipJob J, long n)
{
    const double *s = J.src[blockIdx.y];
    double *d = J.dst[blockIdx.y];
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        d[e] = 1.0 / s[e];
}

__global__ void k_delta_tables(const double *__restrict__ dip, const double *__restrict__ djp,
                               const double *__restrict__ rp, long n2, const double *__restrict__ dkp,
                               long n1, double *__restrict__ d2, double *__restrict__ d1)
{
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n2; e += (long)gridDim.x * blockDim.x) {
        d2[e] = pow(dip[e] * djp[e] * rp[e], .33333333);
        if (e < n1) d1[e] = pow(dkp[e], .33333333);
    }
}

// ---- red-black SOR half sweep ---------------------------------------------
// Points with (i + j + k) % 2 == color are updated; the others are read.
template <typename T>
__global__ void __launch_bounds__(256) k_rb(const BlkDev *__restrict__ blk, int color, T omega,
                                            const T *__restrict__ E, const T *__restrict__ N,
                                            const T *__restrict__ R, const T *__restrict__ D,
                                            T *__restrict__ x, const T *__restrict__ bb,
                                            const PushDev *__restrict__ push)
{
    const BlkDev b = blk[blockIdx.y];
    int ni = b.n[0] - 2, nj = b.n[1] - 2, nk = b.n[2] - 2;
    int nh = (ni + 1) >> 1;
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)nh * nj * nk) return;
    long t = q / nh;
    int ii = (int)(q - t * nh);
    int k = (int)(t / nj) + 2;
    int j = (int)(t - (long)(k - 2) * nj) + 2;
    int i = 2 + 2 * ii + ((2 + j + k + color) & 1);
    if (i > ni + 1) return;
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    long p = b.off3 + (i - 1) + jo * (j - 1) + ko * (k - 1);
    T s = bb[p] + E[p - 1] * x[p - 1] + E[p] * x[p + 1] + N[p - jo] * x[p - jo] +
          N[p] * x[p + jo] + R[p - ko] * x[p - ko] + R[p] * x[p + ko];
    T xo = x[p];
    T xn = xo + omega * (s * D[p] - xo);
    x[p] = xn;
    if (push) push_ghosts(push + 6 * blockIdx.y, b, i, j, k, xn, x);
}

// ---- residual + restriction ------------------------------------------------
// One coarse interior point per thread: the residuals of its 2x2x2 fine
// children are summed into the coarse right-hand side.
template <typename T>
__global__ void __launch_bounds__(256) k_resid_restrict(
    const BlkDev *__restrict__ bc_, const BlkDev *__restrict__ bf_, const T *__restrict__ E,
    const T *__restrict__ N, const T *__restrict__ R, const T *__restrict__ D,
    const T *__restrict__ x, const T *__restrict__ bb, T *__restrict__ bcoarse)
{
    const BlkDev c = bc_[blockIdx.y], f = bf_[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= c.ncell) return;
    int i, j, k;
    long pc = decode_interior(c, q, i, j, k);
    long jo = f.n[0], ko = (long)f.n[0] * f.n[1];
    long p0 = f.off3 + (2 * i - 3) + jo * (2 * j - 3) + ko * (2 * k - 3);
    T sum = 0;
#pragma unroll
    for (int dz = 0; dz < 2; dz++)
#pragma unroll
        for (int dy = 0; dy < 2; dy++)
#pragma unroll
            for (int dx = 0; dx < 2; dx++) {
                long p = p0 + dx + jo * dy + ko * dz;
                T ax = E[p - 1] * x[p - 1] + E[p] * x[p + 1] + N[p - jo] * x[p - jo] +
                       N[p] * x[p + jo] + R[p - ko] * x[p - ko] + R[p] * x[p + ko];
                sum += bb[p] - x[p] / D[p] + ax;
            }
    bcoarse[pc] = sum;
}

// ---- prolongation + correction --------------------------------------------
template <typename T>
__device__ __forceinline__ int clamp_c(int ic, int n, int lo_int, int hi_int)
{
    if (ic == 1 && !lo_int) return 2;
    if (ic == n && !hi_int) return n - 1;
    return ic;
}

template <typename T>
__global__ void __launch_bounds__(256) k_prolong(const BlkDev *__restrict__ bc_,
                                                 const BlkDev *__restrict__ bf_,
                                                 const T *__restrict__ xc, T *__restrict__ xf,
                                                 const PushDev *__restrict__ push)
{
    const BlkDev c = bc_[blockIdx.y], f = bf_[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= f.ncell) return;
    int i, j, k;
    long pf = decode_interior(f, q, i, j, k);
    int ic = (i + 1) >> 1, a = (i + 1) & 1;
    int jc = (j + 1) >> 1, bq = (j + 1) & 1;
    int kc = (k + 1) >> 1, cq = (k + 1) & 1;
    const T w[4] = {(T)0.421875, (T)0.140625, (T)0.046875, (T)0.015625};
    bool iw = c.bc[0] == LES_BCT_INTERFACE_D, ie = c.bc[1] == LES_BCT_INTERFACE_D;
    bool js = c.bc[2] == LES_BCT_INTERFACE_D, jn = c.bc[3] == LES_BCT_INTERFACE_D;
    bool kl = c.bc[4] == LES_BCT_INTERFACE_D, kr = c.bc[5] == LES_BCT_INTERFACE_D;
    long joc = c.n[0], koc = (long)c.n[0] * c.n[1];
    T cr = 0;
#pragma unroll
    for (int sz = 0; sz < 2; sz++)
#pragma unroll
        for (int sy = 0; sy < 2; sy++)
#pragma unroll
            for (int sx = 0; sx < 2; sx++) {
                int h = (sx != a) + (sy != bq) + (sz != cq);
                int ii = clamp_c<T>(ic + sx, c.n[0], iw, ie);
                int jj = clamp_c<T>(jc + sy, c.n[1], js, jn);
                int kk = clamp_c<T>(kc + sz, c.n[2], kl, kr);
                cr += w[h] * xc[c.off3 + (ii - 1) + joc * (jj - 1) + koc * (kk - 1)];
            }
    T v = xf[pf] + cr;
    xf[pf] = v;
    if (push) push_ghosts(push + 6 * blockIdx.y, f, i, j, k, v, xf);
}

// ---- halo for the fast solvers ---------------------------------------------
// Direct copy partner plane -> own ghost plane, face interiors only: the
// 7-point operator never reads edge or corner ghosts, and leaving them out
// makes the copy free of read/write overlaps between faces.
template <typename T>
__global__ void k_halo_fast(const FaceDev *__restrict__ fc, T *__restrict__ x)
{
    const FaceDev f = fc[blockIdx.y];
    long nj = f.nj - 2, nk = f.nk - 2;
    long n = nj * nk;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        long k = q / nj + 1, j = q - (k - 1) * nj + 1;
        x[f.gh + f.jo * j + f.ko * k] = x[f.ppk + f.pjo * j + f.pko * k];
    }
}

// ---- outer FP64 residual (defect correction) -------------------------------
// r = b - A p with the exact FP64 coefficients; writes r (as T) as the
// right-hand side of the next correction cycle and partial sums of r^2 and
// b^2 for the stop test.  `shift` (nullable, device scalar) is subtracted
// from b first: the interior mean of b for a singular operator.
template <typename T>
__global__ void __launch_bounds__(256) k_resid_outer(
    const BlkDev *__restrict__ blk, const double *__restrict__ E, const double *__restrict__ N,
    const double *__restrict__ R, const double *__restrict__ P, const double *__restrict__ x,
    const double *__restrict__ bb, const double *__restrict__ shift, T *__restrict__ rT,
    double *__restrict__ partial)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    double v[2] = {0., 0.};
    const double s0 = shift ? *shift : 0.;
    for (; q < b.ncell; q += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        long p = decode_interior(b, q, i, j, k);
        long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
        const double bp = bb[p] - s0;
        double r = bp - P[p] * x[p] + E[p - 1] * x[p - 1] + E[p] * x[p + 1] +
                   N[p - jo] * x[p - jo] + N[p] * x[p + jo] + R[p - ko] * x[p - ko] +
                   R[p] * x[p + ko];
        rT[p] = (T)r;
        v[0] += r * r;
        v[1] += bp * bp;
    }
    block_reduce_store<2>(v, partial + 2 * (blockIdx.y * (long)gridDim.x + blockIdx.x));
}

__global__ void k_sum2_final(const double *__restrict__ partial, long nparts, double *__restrict__ out)
{
    double v[2] = {0., 0.};
    for (long t = threadIdx.x; t < nparts; t += blockDim.x) {
        v[0] += partial[2 * t];
        v[1] += partial[2 * t + 1];
    }
    __shared__ double r[2];
    block_reduce_store<2>(v, r);
    __syncthreads();
    if (threadIdx.x == 0) {
        out[0] = r[0];
        out[1] = r[1];
    }
}

// Interior mean of a level-1 FP64 field over all blocks.  For a singular
// operator (no Dirichlet side anywhere) the constant vector spans the null
// space of the symmetric coeff_p matrix, so b minus this mean is the part
// of the right-hand side that any p can match; the fast solvers drive the
// residual of that compatible part.
__global__ void __launch_bounds__(256) k_interior_sum(const BlkDev *__restrict__ blk,
                                                      const double *__restrict__ bb,
                                                      double *__restrict__ partial)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    double v[1] = {0.};
    for (; q < b.ncell; q += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        v[0] += bb[decode_interior(b, q, i, j, k)];
    }
    block_reduce_store<1>(v, partial + blockIdx.y * (long)gridDim.x + blockIdx.x);
}

__global__ void k_mean_final(const double *__restrict__ partial, long nparts, double ncell,
                             double *__restrict__ out)
{
    double v[1] = {0.};
    for (long t = threadIdx.x; t < nparts; t += blockDim.x) v[0] += partial[t];
    __shared__ double r[1];
    block_reduce_store<1>(v, r);
    __syncthreads();
    if (threadIdx.x == 0) out[0] = r[0] / ncell;
}

// Coarsest level of a singular (pure Neumann / periodic) operator: remove
// the mean of the right-hand side over all interior points so the coarse
// problem is compatible and its smoothing cannot drift along the constant
// null vector.  One CTA; the level has a few hundred points at most.
template <typename T>
__global__ void k_coarse_mean(const BlkDev *__restrict__ blk, int nb, T *__restrict__ bb)
{
    double v[2] = {0., 0.};
    for (int ib = 0; ib < nb; ib++) {
        const BlkDev b = blk[ib];
        for (long q = threadIdx.x; q < b.ncell; q += blockDim.x) {
            int i, j, k;
            long p = decode_interior(b, q, i, j, k);
            v[0] += (double)bb[p];
            v[1] += 1.0;
        }
    }
    __shared__ double tot[2];
    block_reduce_store<2>(v, tot);
    __syncthreads();
    T mean = (T)(tot[0] / tot[1]);
    for (int ib = 0; ib < nb; ib++) {
        const BlkDev b = blk[ib];
        for (long q = threadIdx.x; q < b.ncell; q += blockDim.x) {
            int i, j, k;
            long p = decode_interior(b, q, i, j, k);
            bb[p] -= mean;
        }
    }
}

// p += e on the interior of level 1
template <typename T>
__global__ void k_update(const BlkDev *__restrict__ blk, double *__restrict__ p,
                         const T *__restrict__ e, const PushDev *__restrict__ push)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long pp = decode_interior(b, q, i, j, k);
    double v = p[pp] + (double)e[pp];
    p[pp] = v;
    if (push) push_ghosts(push + 6 * blockIdx.y, b, i, j, k, v, p);
}

// ================================================================ launchers
namespace les {

static inline unsigned nb_(long n, int t) { return (unsigned)((n + t - 1) / t); }

template <typename T>
int launch_conv_coef(const BlkDev *blk, int nb, long maxcell, const double *const *a, T *E, T *N,
                     T *R, T *D, double *E64, double *N64, double *R64, double *P64, int *bad,
                     cudaStream_t st)
{
    k_conv_coef<T><<<dim3(nb_(maxcell, 128), nb), 128, 0, st>>>(blk, a[0], a[1], a[2], a[3], a[4], a[5],
                                                               a[6], E, N, R, D, E64, N64, R64, P64,
                                                               bad);
    count_launch(1);
    return 0;
}

// maxhalf = max over blocks of ((ni + 1) / 2) * nj * nk
template <typename T>
void launch_rb(const BlkDev *blk, int nb, long maxhalf, int color, double omega, const T *E,
               const T *N, const T *R, const T *D, T *x, const T *b, const PushDev *push,
               cudaStream_t st)
{
    k_rb<T><<<dim3(nb_(maxhalf, 256), nb), 256, 0, st>>>(blk, color, (T)omega, E, N, R, D, x, b, push);
    count_launch(1);
}

template <typename T>
void launch_resid_restrict(const BlkDev *bc, const BlkDev *bf, int nb, long maxcell_c, const T *E,
                           const T *N, const T *R, const T *D, const T *x, const T *b, T *bcoarse,
                           cudaStream_t st)
{
    k_resid_restrict<T><<<dim3(nb_(maxcell_c, 256), nb), 256, 0, st>>>(bc, bf, E, N, R, D, x, b,
                                                                     bcoarse);
    count_launch(1);
}

template <typename T>
void launch_prolong_fast(const BlkDev *bc, const BlkDev *bf, int nb, long maxcell_f, const T *xc,
                         T *xf, const PushDev *push, cudaStream_t st)
{
    k_prolong<T><<<dim3(nb_(maxcell_f, 256), nb), 256, 0, st>>>(bc, bf, xc, xf, push);
    count_launch(1);
}

template <typename T>
void launch_halo_fast(const FaceDev *faces, int nface, long maxface, T *x, cudaStream_t st)
{
    if (nface == 0) return;
    unsigned gx = nb_(maxface, 256);
    if (gx > 32) gx = 32;
    k_halo_fast<T><<<dim3(gx, nface), 256, 0, st>>>(faces, x);
    count_launch(1);
}

template <typename T>
void launch_resid_outer(const BlkDev *blk, int nb, long maxcell, const double *E, const double *N,
                        const double *R, const double *P, const double *x, const double *b,
                        const double *shift, T *rT, double *partial, double *out2, cudaStream_t st)
{
    // grid-stride: a few CTAs per SM, so the final sum reads few partials
    unsigned gx = nb_(maxcell, 256);
    unsigned cap = (unsigned)((1216 + nb - 1) / nb);
    if (gx > cap) gx = cap;
    k_resid_outer<T><<<dim3(gx, nb), 256, 0, st>>>(blk, E, N, R, P, x, b, shift, rT, partial);
    k_sum2_final<<<1, 256, 0, st>>>(partial, (long)gx * nb, out2);
    count_launch(2);
}

void launch_interior_mean(const BlkDev *blk, int nb, long maxcell, const double *b, double ncell,
                          double *partial, double *out, cudaStream_t st)
{
    unsigned gx = nb_(maxcell, 256);
    unsigned cap = (unsigned)((1216 + nb - 1) / nb);
    if (gx > cap) gx = cap;
    k_interior_sum<<<dim3(gx, nb), 256, 0, st>>>(blk, b, partial);
    k_mean_final<<<1, 256, 0, st>>>(partial, (long)gx * nb, ncell, out);
    count_launch(2);
}

void launch_recip(const double *const *src, double *const *dst, int ntab, long n, cudaStream_t st)
{
    RecipJob J;
    for (int b0 = 0; b0 < ntab; b0 += 24) {
        int m = ntab - b0 < 24 ? ntab - b0 : 24;
        for (int t = 0; t < m; t++) {
            J.src[t] = src[b0 + t];
            J.dst[t] = dst[b0 + t];
        }
        unsigned gx = nb_(n, 256);
        if (gx > 256) gx = 256;
        k_recip<<<dim3(gx, m), 256, 0, st>>>(J, n);
        count_launch(1);
    }
}

void launch_delta_tables(const double *dip, const double *djp, const double *rp, long n2,
                         const double *dkp, long n1, double *d2, double *d1, cudaStream_t st)
{
    long n = n2 > n1 ? n2 : n1;
    unsigned gx = nb_(n, 256);
    if (gx > 1024) gx = 1024;
    k_delta_tables<<<gx, 256, 0, st>>>(dip, djp, rp, n2, dkp, n1, d2, d1);
    count_launch(1);
}

template <typename T>
void launch_coarse_mean(const BlkDev *blk, int nb, T *b, cudaStream_t st)
{
    k_coarse_mean<T><<<1, 512, 0, st>>>(blk, nb, b);
    count_launch(1);
}

template <typename T>
void launch_update(const BlkDev *blk, int nb, long maxcell, double *p, const T *e, const PushDev *push,
                   cudaStream_t st)
{
    k_update<T><<<dim3(nb_(maxcell, 256), nb), 256, 0, st>>>(blk, p, e, push);
    count_launch(1);
}

#define INST(T)                                                                                    \
    template int launch_conv_coef<T>(const BlkDev *, int, long, const double *const *, T *, T *,   \
                                     T *, T *, double *, double *, double *, double *, int *,     \
                                     cudaStream_t);                                                \
    template void launch_rb<T>(const BlkDev *, int, long, int, double, const T *, const T *,      \
                               const T *, const T *, T *, const T *, const PushDev *,             \
                               cudaStream_t);                                                     \
    template void launch_resid_restrict<T>(const BlkDev *, const BlkDev *, int, long, const T *,  \
                                           const T *, const T *, const T *, const T *, const T *, \
                                           T *, cudaStream_t);                                    \
    template void launch_prolong_fast<T>(const BlkDev *, const BlkDev *, int, long, const T *,    \
                                         T *, const PushDev *, cudaStream_t);                     \
    template void launch_halo_fast<T>(const FaceDev *, int, long, T *, cudaStream_t);             \
    template void launch_resid_outer<T>(const BlkDev *, int, long, const double *,                \
                                        const double *, const double *, const double *,           \
                                        const double *, const double *, const double *, T *,      \
                                        double *, double *, cudaStream_t);                        \
    template void launch_update<T>(const BlkDev *, int, long, double *, const T *, const PushDev *, \
                                   cudaStream_t);                                                \
    template void launch_coarse_mean<T>(const BlkDev *, int, T *, cudaStream_t);
INST(float)
INST(double)
#undef INST

} // namespace les
