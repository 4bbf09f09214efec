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
#include <algorithm>

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
    pdl_wait();
    pdl_trigger();
    const double *s = J.src[blockIdx.y];
    double *d = J.dst[blockIdx.y];
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        d[e] = 1.0 / s[e];
}

// FP32 copies of FP64 tables (the FP32 physics build's metrics)
struct F32Job {
    const double *src[24];
    float *dst[24];
};

__global__ void k_to_f32(F32Job J, long n)
{
    pdl_wait();
    pdl_trigger();
    const double *s = J.src[blockIdx.y];
    float *d = J.dst[blockIdx.y];
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        d[e] = (float)s[e];
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

// 1 / v correctly rounded, the value of (T)1 / v (IEEE division), from the
// reciprocal intrinsic without the division's numerator scaling
__device__ __forceinline__ float rcp_rn(float v) { return __frcp_rn(v); }
__device__ __forceinline__ double rcp_rn(double v) { return __drcp_rn(v); }

// ---- separable (matrix-free) coefficients ---------------------------------
// coeff_p's couplings factor into a 2-D (i, j) part and a 1-D k part
// (code/coeff_p_block.F: ae = rdju/diu * dkp(k), an = rdiv/djv * dkp(k),
// ar = didjp/rp / dkw(k+1), with the boundary rows zeroed or recomputed per
// (i, j) or per k).  The FP32 solver then needs no coefficient arrays: the
// factors are taken from the converted coefficients at a reference column
// and point of each block, checked against every coefficient
// (k_mf_check), and the six couplings and 1/ap are formed on the fly.
template <typename T>
__device__ __forceinline__ void coefs_mf(const BlkDev &b, const MfTab<T> &t, int i, int j, int k,
                                         T c[6], T &dinv)
{
    const long n0 = b.n[0];
    const long ij = b.off2 + (i - 1) + n0 * (j - 1), kk = b.off1k + (k - 1);
    const T ez = t.Ez[kk], nz = t.Nz[kk], r2 = t.R2[ij];
    c[0] = t.E2[ij - 1] * ez;
    c[1] = t.E2[ij] * ez;
    c[2] = t.N2[ij - n0] * nz;
    c[3] = t.N2[ij] * nz;
    c[4] = r2 * t.Rz[kk - 1];
    c[5] = r2 * t.Rz[kk];
    dinv = rcp_rn((((c[0] + c[1]) + (c[2] + c[3])) + (c[4] + c[5])));
}

// 2-D factors at k = kr, 1-D factors along the reference column (i0, j0)
template <typename T>
__global__ void k_mf_extract(const BlkDev *__restrict__ blk, const T *__restrict__ E,
                             const T *__restrict__ N, const T *__restrict__ R, MfTab<T> t,
                             int *__restrict__ bad)
{
    const BlkDev b = blk[blockIdx.y];
    const int n0 = b.n[0], n1 = b.n[1], n2 = b.n[2];
    const long jo = n0, ko = (long)n0 * n1;
    const int i0 = (n0 + 1) / 2, j0 = (n1 + 1) / 2, kr = (n2 + 1) / 2;
    const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q < (long)n0 * n1) {
        long p = b.off3 + q + ko * (kr - 1);
        t.E2[b.off2 + q] = E[p];
        t.N2[b.off2 + q] = N[p];
        t.R2[b.off2 + q] = R[p];
    }
    if (q < n2) {
        long pc = b.off3 + (i0 - 1) + jo * (j0 - 1);
        T e0 = E[pc + ko * (kr - 1)], nn0 = N[pc + ko * (kr - 1)], r0 = R[pc + ko * (kr - 1)];
        if (e0 == (T)0 || nn0 == (T)0 || r0 == (T)0) {
            atomicOr(bad, 16);
            return;
        }
        t.Ez[b.off1k + q] = E[pc + ko * q] / e0;
        t.Nz[b.off1k + q] = N[pc + ko * q] / nn0;
        t.Rz[b.off1k + q] = R[pc + ko * q] / r0;
    }
}

// every coupling and ap of every interior point within tol * ap
template <typename T>
__global__ void k_mf_check(const BlkDev *__restrict__ blk, const T *__restrict__ E,
                           const T *__restrict__ N, const T *__restrict__ R,
                           const T *__restrict__ D, MfTab<T> t, T tol, int *__restrict__ bad)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long p = decode_interior(b, q, i, j, k);
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    T c[6], dinv;
    coefs_mf(b, t, i, j, k, c, dinv);
    const T ref[6] = {E[p - 1], E[p], N[p - jo], N[p], R[p - ko], R[p]};
    const T ap = (T)1 / D[p];
    bool ok = fabs((double)(1 / dinv) - (double)ap) <= (double)tol * fabs((double)ap);
    for (int m = 0; m < 6; m++) ok = ok && fabs((double)(c[m] - ref[m])) <= (double)tol * fabs((double)ap);
    if (!ok) atomicOr(bad, 32);
}

// ---- red-black SOR half sweep ---------------------------------------------
// Points with (i + j + k) % 2 == color are updated; the others are read.
// one red-black update of interior point (i, j, k) of block bi
template <typename T>
__device__ __forceinline__ void rb_point(const BlkDev &b, int bi, int i, int j, int k, T omega,
                                         const T *__restrict__ E, const T *__restrict__ N,
                                         const T *__restrict__ R, const T *__restrict__ D,
                                         T *__restrict__ x, const T *__restrict__ bb,
                                         const PushDev *__restrict__ push, const MfTab<T> &mf)
{
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    long p = b.off3 + (i - 1) + jo * (j - 1) + ko * (k - 1);
    T c[6], dinv;
    if (mf.E2) {
        coefs_mf(b, mf, i, j, k, c, dinv);
    } else {
        c[0] = E[p - 1];
        c[1] = E[p];
        c[2] = N[p - jo];
        c[3] = N[p];
        c[4] = R[p - ko];
        c[5] = R[p];
        dinv = D[p];
    }
    T s = bb[p] + c[0] * x[p - 1] + c[1] * x[p + 1] + c[2] * x[p - jo] + c[3] * x[p + jo] +
          c[4] * x[p - ko] + c[5] * x[p + ko];
    T xo = x[p];
    T xn = xo + omega * (s * dinv - xo);
    x[p] = xn;
    if (push) push_ghosts(push + 6 * bi, b, i, j, k, xn, x);
}

// thread q of a half sweep of colour `color` -> point (i, j, k); false if none
__device__ __forceinline__ bool rb_decode(const BlkDev &b, unsigned q, int color, int &i, int &j, int &k)
{
    const int ni = b.n[0] - 2, nj = b.n[1] - 2, nk = b.n[2] - 2;
    const unsigned nh = (unsigned)(ni + 1) >> 1;
    if (q >= nh * (unsigned)nj * (unsigned)nk) return false;
    const unsigned t = q / nh;
    const int ii = (int)(q - t * nh);
    const unsigned tk = t / (unsigned)nj;
    k = (int)tk + 2;
    j = (int)(t - tk * (unsigned)nj) + 2;
    i = 2 + 2 * ii + ((2 + j + k + color) & 1);
    return i <= ni + 1;
}

// ---- red-black SOR half sweep, all blocks of a level ----------------------
// Thread (x, y) of CTA (bx, by, bz): point 2 + 2 (32 bx + x) (+1 by colour)
// of row j = 2 + blockDim.y by + y of the (block, plane) zmap[z0 + bz]; no
// per-thread division.  Ix: the offset type, int when every
// offset of the multigrid arrays is below 2^31.  Per point the operations
// of rb_point.
// One point of a half sweep at offset p (ij, kk: its 2-D and 1-D table
// offsets; jo, ko: its block's strides): the couplings (separable factors
// or arrays), then -- once the kernel before has finished -- the update
// x[p] = x + omega (s / ap - x); returns the new value.  rb_point's
// operations in the same order.
template <typename T, bool MF, typename Ix>
__device__ __forceinline__ T rb_update(Ix p, Ix ij, Ix kk, Ix jo, Ix ko, T omega, const T *__restrict__ E,
                                       const T *__restrict__ N, const T *__restrict__ R, const T *__restrict__ D,
                                       T *__restrict__ x, const T *__restrict__ bb, const MfTab<T> &mf)
{
    T c[6], dinv;
    if (MF) {
        const T ez = mf.Ez[kk], nz = mf.Nz[kk], r2 = mf.R2[ij];
        c[0] = mf.E2[ij - 1] * ez;
        c[1] = mf.E2[ij] * ez;
        c[2] = mf.N2[ij - jo] * nz;
        c[3] = mf.N2[ij] * nz;
        c[4] = r2 * mf.Rz[kk - 1];
        c[5] = r2 * mf.Rz[kk];
        dinv = rcp_rn((((c[0] + c[1]) + (c[2] + c[3])) + (c[4] + c[5])));
    } else {
        c[0] = E[p - 1];
        c[1] = E[p];
        c[2] = N[p - jo];
        c[3] = N[p];
        c[4] = R[p - ko];
        c[5] = R[p];
        dinv = D[p];
    }
    pdl_wait();
    pdl_trigger();
    const T *xp = x + p;
    T s = bb[p] + c[0] * xp[-1] + c[1] * xp[1] + c[2] * xp[-jo] + c[3] * xp[jo] + c[4] * xp[-ko] + c[5] * xp[ko];
    T xo = xp[0];
    T xn = xo + omega * (s * dinv - xo);
    x[p] = xn;
    return xn;
}

template <typename T, bool MF, typename Ix>
__global__ void __launch_bounds__(512) k_rb(const BlkDev *__restrict__ blk, int color, T omega,
                                            const T *__restrict__ E, const T *__restrict__ N,
                                            const T *__restrict__ R, const T *__restrict__ D,
                                            T *__restrict__ x, const T *__restrict__ bb,
                                            const PushDev *__restrict__ push, MfTab<T> mf,
                                            const int2 *__restrict__ zmap, int z0)
{
    const int2 bk = zmap[z0 + blockIdx.z];
    const int bi = bk.x, k = bk.y;
    const int n0 = blk[bi].n[0], n1 = blk[bi].n[1], n2 = blk[bi].n[2];
    const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y) + 2;
    if (k > n2 - 1 || j > n1 - 1) return;
    const int i = 2 + 2 * (int)(blockIdx.x * 32 + threadIdx.x) + ((j + k + color) & 1);
    if (i > n0 - 1) return;
    const Ix jo = n0, ko = (Ix)n0 * n1;
    const Ix p = (Ix)blk[bi].off3 + (i - 1) + jo * (j - 1) + ko * (k - 1);
    const Ix ij = (Ix)blk[bi].off2 + (i - 1) + jo * (j - 1), kk = (Ix)blk[bi].off1k + (k - 1);
    const T xn = rb_update<T, MF, Ix>(p, ij, kk, jo, ko, omega, E, N, R, D, x, bb, mf);
    if (push && (i == 2 || i == n0 - 1 || j == 2 || j == n1 - 1 || k == 2 || k == n2 - 1))
        push_ghosts(push + 6 * bi, blk[bi], i, j, k, xn, x);
}

// The same half sweep with the level's geometry as a kernel parameter
// (LevGeo): no descriptor loads, and for one block no division either.
// PUSH: some face of the level mirrors its first interior plane.
template <typename T, bool MF, bool ONE, bool PUSH>
__global__ void __launch_bounds__(512) k_rb_geo(const __grid_constant__ LevGeo G, int color, T omega,
                                                const T *__restrict__ E, const T *__restrict__ N,
                                                const T *__restrict__ R, const T *__restrict__ D,
                                                T *__restrict__ x, const T *__restrict__ bb, MfTab<T> mf,
                                                const int2 *__restrict__ zmap)
{
    // one block: plane 2 + bz; several: the (block, plane) map
    int bi = 0, k = (int)blockIdx.z + 2;
    if (!ONE) {
        const int2 bk = zmap[blockIdx.z];
        bi = bk.x;
        k = bk.y;
    }
    const int n0 = G.n[bi][0], n1 = G.n[bi][1], n2 = G.n[bi][2];
    const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y) + 2;
    if (k > n2 - 1 || j > n1 - 1) return;
    const int i = 2 + 2 * (int)(blockIdx.x * 32 + threadIdx.x) + ((j + k + color) & 1);
    if (i > n0 - 1) return;
    const int jo = n0, ko = n0 * n1;
    const int p = G.off3[bi] + (i - 1) + jo * (j - 1) + ko * (k - 1);
    const int ij = G.off2[bi] + (i - 1) + jo * (j - 1), kk = G.off1k[bi] + (k - 1);
    const T xn = rb_update<T, MF, int>(p, ij, kk, jo, ko, omega, E, N, R, D, x, bb, mf);
    if (PUSH && (i == 2 || i == n0 - 1 || j == 2 || j == n1 - 1 || k == 2 || k == n2 - 1)) {
        // push_ghosts with the mirrors from the parameter
        const int cc[3] = {i - 1, j - 1, k - 1}, nn[3] = {n0, n1, n2};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            if (cc[d] == 1 && G.push[bi][2 * d].valid) {
                const PushDev &P = G.push[bi][2 * d];
                x[P.gh + P.jo * cc[P.a2] + P.ko * cc[P.a3]] = xn;
            }
            if (cc[d] == nn[d] - 2 && G.push[bi][2 * d + 1].valid) {
                const PushDev &P = G.push[bi][2 * d + 1];
                x[P.gh + P.jo * cc[P.a2] + P.ko * cc[P.a3]] = xn;
            }
        }
    }
}

// ---- red-black SOR, one full sweep per launch, shared-memory tiles --------
// For a level of one block whose faces are periodic onto itself with even
// extents, or walls (no coupling through them): each CTA stages a tile of
// kTI x kTJ x kTK points of x with a two-point halo and of b with a
// one-point halo (periodic axes wrapped, the wall sides clamped: their
// couplings are zero), updates colour 0 on the tile and its one-point halo,
// then colour 1 on the tile, in shared memory, and writes the tile to the
// other buffer (with the ghosts its boundary points mirror).  The halo's
// colour-0 values are recomputed from the same staged values the
// neighbouring tile uses, so the sweep is the two half sweeps of k_rb, per
// point the same operations; x is read once per sweep instead of twice and
// one launch replaces two.
constexpr int kTI = 32, kTJ = 16, kTK = 8;
constexpr int kXI = kTI + 4, kXJ = kTJ + 4, kXK = kTK + 4;
constexpr int kBI = kTI + 2, kBJ = kTJ + 2, kBK = kTK + 2;
// separable couplings of the tile and its one-point halo (coefs_mf's
// operands, per (i, j) column and per k)
constexpr int kMf2 = 5 * kBJ * kBI, kMf1 = 4 * kBK;
template <typename T>
constexpr size_t kRbTileSmem = sizeof(T) * (kXK * kXJ * kXI + kBK * kBJ * kBI + kMf2 + kMf1);

// the source of unwrapped coordinate c on an axis with interior 2..n+1:
// wrapped on a periodic axis, clamped to the ghosts 1..n+2 otherwise
__device__ __forceinline__ int rbt_src(int c, int n, bool per)
{
    if (per) return c < 2 ? c + n : c > n + 1 ? c - n : c;
    return c < 1 ? 1 : c > n + 2 ? n + 2 : c;
}

// one element, global -> shared, asynchronously (cp.async; completes at
// the CTA's wait_group)
template <typename T> __device__ __forceinline__ void rbt_async(T *dst, const T *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}

template <typename T>
__global__ void __launch_bounds__(256) k_rb_tile(const BlkDev *__restrict__ blk, T omega, const T *__restrict__ xin,
                                                 T *__restrict__ xout, const T *__restrict__ bb,
                                                 const PushDev *__restrict__ push, MfTab<T> mf)
{
    extern __shared__ __align__(16) unsigned char rbt_smem[];
    T *const X = (T *)rbt_smem;
    T *const Bs = X + kXK * kXJ * kXI;
    T *const M2 = Bs + kBK * kBJ * kBI;  // [5][kBJ][kBI]: E2 west, E2, N2 south, N2, R2
    T *const M1 = M2 + kMf2;             // [4][kBK]: Ez, Nz, Rz below, Rz
    const BlkDev b = blk[0];
    const int ni = b.n[0] - 2, nj = b.n[1] - 2, nk = b.n[2] - 2;
    const bool pi = b.bc[0] == LES_BCT_PERIODIC_D, pj = b.bc[2] == LES_BCT_PERIODIC_D,
               pk = b.bc[4] == LES_BCT_PERIODIC_D;
    const int ntx = (ni + kTI - 1) / kTI, nty = (nj + kTJ - 1) / kTJ;
    const int t = blockIdx.x, tx = t % ntx, ty = (t / ntx) % nty, tz = t / (ntx * nty);
    const int i0 = 2 + kTI * tx, j0 = 2 + kTJ * ty, k0 = 2 + kTK * tz;
    const long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    // staging, a warp per row (lanes along i), as asynchronous copies
    // (cp.async) all in flight at once, then one wait
    for (int r = warp; r < kXJ * kXK; r += nwarp) {
        const int bq = r % kXJ, cq = r / kXJ;
        const long row = b.off3 - 1 + jo * (rbt_src(j0 - 2 + bq, nj, pj) - 1) + ko * (rbt_src(k0 - 2 + cq, nk, pk) - 1);
        for (int a = lane; a < kXI; a += 32) rbt_async(&X[r * kXI + a], xin + row + rbt_src(i0 - 2 + a, ni, pi));
    }
    for (int r = warp; r < kBJ * kBK; r += nwarp) {
        const int bq = r % kBJ, cq = r / kBJ;
        const long row = b.off3 - 1 + jo * (rbt_src(j0 - 1 + bq, nj, pj) - 1) + ko * (rbt_src(k0 - 1 + cq, nk, pk) - 1);
        for (int a = lane; a < kBI; a += 32) rbt_async(&Bs[r * kBI + a], bb + row + rbt_src(i0 - 1 + a, ni, pi));
    }
    {
        const long n0 = b.n[0];
        // positions outside the level (clamped on a physical side) are
        // never updated: zeros there, and no read outside the tables
        for (int e = threadIdx.x; e < kBJ * kBI; e += blockDim.x) {
            const int a = e % kBI, bq = e / kBI;
            const int iw = rbt_src(i0 - 1 + a, ni, pi), jw = rbt_src(j0 - 1 + bq, nj, pj);
            if (iw < 2 || iw > ni + 1 || jw < 2 || jw > nj + 1) {
                for (int f = 0; f < 5; f++) M2[f * kBJ * kBI + e] = (T)0;
                continue;
            }
            const long ij = b.off2 + (iw - 1) + n0 * (jw - 1);
            rbt_async(&M2[e], mf.E2 + ij - 1);
            rbt_async(&M2[kBJ * kBI + e], mf.E2 + ij);
            rbt_async(&M2[2 * kBJ * kBI + e], mf.N2 + ij - n0);
            rbt_async(&M2[3 * kBJ * kBI + e], mf.N2 + ij);
            rbt_async(&M2[4 * kBJ * kBI + e], mf.R2 + ij);
        }
        for (int e = threadIdx.x; e < kBK; e += blockDim.x) {
            const int kw = rbt_src(k0 - 1 + e, nk, pk);
            if (kw < 2 || kw > nk + 1) {
                for (int f = 0; f < 4; f++) M1[f * kBK + e] = (T)0;
                continue;
            }
            const long kk = b.off1k + (kw - 1);
            rbt_async(&M1[e], mf.Ez + kk);
            rbt_async(&M1[kBK + e], mf.Nz + kk);
            rbt_async(&M1[2 * kBK + e], mf.Rz + kk - 1);
            rbt_async(&M1[3 * kBK + e], mf.Rz + kk);
        }
    }
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    constexpr int sJ = kXI, sK = kXI * kXJ, sM = kBJ * kBI;
    // one update of the staged point at X index xe, b at Bs index be, the
    // couplings from the staged separable factors of column bc and layer
    // bk: coefs_mf's and rb_point's operations
    auto update = [&](int xe, int be, int bc, int bk) {
        const T ez = M1[bk], nz = M1[kBK + bk], r2 = M2[4 * sM + bc];
        const T c0 = M2[bc] * ez, c1 = M2[sM + bc] * ez, c2 = M2[2 * sM + bc] * nz, c3 = M2[3 * sM + bc] * nz;
        const T c4 = r2 * M1[2 * kBK + bk], c5 = r2 * M1[3 * kBK + bk];
        const T dinv = rcp_rn((((c0 + c1) + (c2 + c3)) + (c4 + c5)));
        const T s = Bs[be] + c0 * X[xe - 1] + c1 * X[xe + 1] + c2 * X[xe - sJ] + c3 * X[xe + sJ] + c4 * X[xe - sK] +
                    c5 * X[xe + sK];
        const T xo = X[xe];
        X[xe] = xo + omega * (s * dinv - xo);
    };
    // colour 0 on the tile and its one-point halo, where that is a point of
    // the level (wrapped on periodic axes): a warp per row of the halo box,
    // lane m on its m-th colour-0 point
    for (int r = warp; r < kBJ * kBK; r += nwarp) {
        const int bq = r % kBJ, cq = r / kBJ, j = j0 - 1 + bq, k = k0 - 1 + cq;
        if ((!pj && (j < 2 || j > nj + 1)) || (!pk && (k < 2 || k > nk + 1))) continue;
        const int a = ((i0 - 1 + j + k) & 1) + 2 * lane, i = i0 - 1 + a;
        if (a >= kBI || (!pi && (i < 2 || i > ni + 1))) continue;
        update(((cq + 1) * kXJ + bq + 1) * kXI + a + 1, r * kBI + a, bq * kBI + a, cq);
    }
    __syncthreads();
    // colour 1 on the tile's points of the level: a half warp per tile row
    for (int r = 2 * warp + (lane >> 4); r < kTJ * kTK; r += 2 * nwarp) {
        const int bq = r % kTJ, cq = r / kTJ, j = j0 + bq, k = k0 + cq;
        const int a = ((i0 + j + k + 1) & 1) + 2 * (lane & 15), i = i0 + a;
        if (i > ni + 1 || j > nj + 1 || k > nk + 1) continue;
        update(((cq + 2) * kXJ + bq + 2) * kXI + a + 2, ((cq + 1) * kBJ + bq + 1) * kBI + a + 1,
               (bq + 1) * kBI + a + 1, cq + 1);
    }
    __syncthreads();
    // the tile out, a warp per row, and the ghosts its boundary points mirror
    for (int r = warp; r < kTJ * kTK; r += nwarp) {
        const int bq = r % kTJ, cq = r / kTJ, j = j0 + bq, k = k0 + cq, i = i0 + lane;
        if (i > ni + 1 || j > nj + 1 || k > nk + 1) continue;
        const T v = X[((cq + 2) * kXJ + bq + 2) * kXI + lane + 2];
        xout[b.off3 + (i - 1) + jo * (j - 1) + ko * (k - 1)] = v;
        if (push) push_ghosts(push, b, i, j, k, v, xout);
    }
}

// ---- y-line zebra relaxation ---------------------------------------------
// One thread per (i, k) column with (i + k) % 2 == color: the column's
// tridiagonal system in j (couplings N to j -/+ 1, the i and k neighbours
// at their current values, the ghost rows j = 1 and nj + 2 known) solved by
// the Thomas algorithm through the scratch arrays cp, dp (same layout as
// x), then x += omega (x_line - x).  Strong coupling in y -- cells much
// thinner than they are long, as at stretched walls -- is what point
// smoothing cannot damp and line relaxation removes.
template <typename T>
__global__ void __launch_bounds__(256) k_yline(const BlkDev *__restrict__ blk, int color, T omega,
                                               const T *__restrict__ E, const T *__restrict__ N,
                                               const T *__restrict__ R, const T *__restrict__ D,
                                               T *__restrict__ x, const T *__restrict__ bb, MfTab<T> mf,
                                               T *__restrict__ cp, T *__restrict__ dp)
{
    const BlkDev b = blk[blockIdx.y];
    const int ni = b.n[0] - 2, nj = b.n[1] - 2, nk = b.n[2] - 2;
    const unsigned nh = (unsigned)(ni + 1) >> 1;
    const unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nh * (unsigned)nk) return;
    const unsigned kq = q / nh;
    const int k = (int)kq + 2;
    const int i = 2 + 2 * (int)(q - kq * nh) + ((2 + k + color) & 1);
    if (i > ni + 1) return;
    const long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    const long p0 = b.off3 + (i - 1) + ko * (k - 1);
    T cprev = 0, dprev = 0;
    for (int j = 2; j <= nj + 1; j++) {
        const long p = p0 + jo * (j - 1);
        T c[6], dinv;
        if (mf.E2) {
            coefs_mf(b, mf, i, j, k, c, dinv);
        } else {
            c[0] = E[p - 1];
            c[1] = E[p];
            c[2] = N[p - jo];
            c[3] = N[p];
            c[4] = R[p - ko];
            c[5] = R[p];
            dinv = D[p];
        }
        T rhs = bb[p] + c[0] * x[p - 1] + c[1] * x[p + 1] + c[4] * x[p - ko] + c[5] * x[p + ko];
        T lo = c[2], up = c[3];
        if (j == 2) {
            rhs += lo * x[p - jo];
            lo = 0;
        }
        if (j == nj + 1) {
            rhs += up * x[p + jo];
            up = 0;
        }
        const T m = (T)1 / dinv - lo * cprev;
        const T cj = up / m, dj = (rhs + lo * dprev) / m;
        cp[p] = cj;
        dp[p] = dj;
        cprev = cj;
        dprev = dj;
    }
    T xnext = 0;
    for (int j = nj + 1; j >= 2; j--) {
        const long p = p0 + jo * (j - 1);
        const T xl = dp[p] + cp[p] * xnext;
        xnext = xl;
        const T xo = x[p];
        x[p] = xo + omega * (xl - xo);
    }
}

// ---- y-line zebra relaxation, a warp per line -----------------------------
// The same relaxation as k_yline with the tridiagonal solve spread over the
// 32 lanes of a warp: lane L holds rows [L m, L m + m) of the line (m =
// ceil(nj / 32) <= kLineM), solves all but its last row by the Thomas
// algorithm with three right-hand sides -- the line's own, and unit
// couplings to the last row of lane L-1 and to its own last row -- so every
// row is y + u X(L-1) + w X(L) in the lanes' last-row values X; the last
// rows' equations then form a tridiagonal system of 32 unknowns, one per
// lane, solved by parallel cyclic reduction over warp shuffles (5 steps),
// and each lane substitutes back.  No scratch arrays; 32 lanes per line
// instead of one thread: used where a level has few lines (launch_yline).
// The elimination order differs from k_yline's, so results agree to
// rounding.
constexpr int kLineM = 16;  // rows per lane: lines of up to 512 points

template <typename T>
__global__ void __launch_bounds__(128) k_yline_warp(const BlkDev *__restrict__ blk, int color, T omega,
                                                    const T *__restrict__ E, const T *__restrict__ N,
                                                    const T *__restrict__ R, const T *__restrict__ D,
                                                    T *__restrict__ x, const T *__restrict__ bb, MfTab<T> mf)
{
    const BlkDev b = blk[blockIdx.y];
    const int ni = b.n[0] - 2, nj = b.n[1] - 2, nk = b.n[2] - 2;
    const unsigned nh = (unsigned)(ni + 1) >> 1;
    const unsigned q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // the warp's line
    const int lane = threadIdx.x & 31;
    if (q >= nh * (unsigned)nk) return;  // whole warps leave together
    const unsigned kq = q / nh;
    const int k = (int)kq + 2;
    const int i = 2 + 2 * (int)(q - kq * nh) + ((2 + k + color) & 1);
    if (i > ni + 1) return;
    const long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    const long p0 = b.off3 + (i - 1) + ko * (k - 1);
    const int m = (nj + 31) / 32;
    const int s = lane * m, e = min(s + m, nj), cnt = max(e - s, 0);
    // row r of the line (j = r + 2) as a x(r-1) + bd x(r) + c x(r+1) = d
    auto row = [&](int r, T &a, T &bd, T &c, T &d) {
        const int j = r + 2;
        const long p = p0 + jo * (j - 1);
        T cf[6], dinv;
        if (mf.E2) {
            coefs_mf(b, mf, i, j, k, cf, dinv);
        } else {
            cf[0] = E[p - 1];
            cf[1] = E[p];
            cf[2] = N[p - jo];
            cf[3] = N[p];
            cf[4] = R[p - ko];
            cf[5] = R[p];
            dinv = D[p];
        }
        T rhs = bb[p] + cf[0] * x[p - 1] + cf[1] * x[p + 1] + cf[4] * x[p - ko] + cf[5] * x[p + ko];
        T lo = cf[2], up = cf[3];
        if (j == 2) {
            rhs += lo * x[p - jo];
            lo = 0;
        }
        if (j == nj + 1) {
            rhs += up * x[p + jo];
            up = 0;
        }
        a = -lo;
        bd = (T)1 / dinv;
        c = -up;
        d = rhs;
    };
    // local Thomas on rows s .. e-2 with three right-hand sides
    T cp[kLineM], vy[kLineM], vu[kLineM], vw[kLineM];
    const int nl = cnt - 1;  // rows of the local system
#pragma unroll
    for (int t = 0; t < kLineM; t++) {
        if (t < nl) {
            T a, bd, c, d;
            row(s + t, a, bd, c, d);
            const T at = t > 0 ? a : (T)0;
            const T den = bd - (t > 0 ? at * cp[t - 1] : (T)0);
            const T ct = t < nl - 1 ? c : (T)0;
            const T ru = t == 0 ? -a : (T)0, rw = t == nl - 1 ? -c : (T)0;
            cp[t] = ct / den;
            vy[t] = (d - (t > 0 ? at * vy[t - 1] : (T)0)) / den;
            vu[t] = (ru - (t > 0 ? at * vu[t - 1] : (T)0)) / den;
            vw[t] = (rw - (t > 0 ? at * vw[t - 1] : (T)0)) / den;
        }
    }
#pragma unroll
    for (int t = kLineM - 2; t >= 0; t--) {
        if (t < nl - 1) {
            vy[t] -= cp[t] * vy[t + 1];
            vu[t] -= cp[t] * vu[t + 1];
            vw[t] -= cp[t] * vw[t + 1];
        }
    }
    // x(s) = F and x(e-2) = G in (X(L-1), X(L)); a one-row lane is X itself
    T fy = 0, fu = 0, fw = 1, gy = 0, gu = 1, gw = 0;
    if (nl > 0) {
        fy = vy[0];
        fu = vu[0];
        fw = vw[0];
#pragma unroll
        for (int t = 0; t < kLineM; t++)
            if (t == nl - 1) {
                gy = vy[t];
                gu = vu[t];
                gw = vw[t];
            }
    }
    const T ny = __shfl_down_sync(0xffffffffu, fy, 1), nu = __shfl_down_sync(0xffffffffu, fu, 1),
            nw = __shfl_down_sync(0xffffffffu, fw, 1);
    const int ncnt = __shfl_down_sync(0xffffffffu, cnt, 1);
    // the reduced equation of the lane's last row
    T A = 0, B = 1, C = 0, Dr = 0;
    if (cnt > 0) {
        T a, bd, c, d;
        row(e - 1, a, bd, c, d);
        const bool nxt = lane < 31 && ncnt > 0;
        const T fyn = nxt ? ny : (T)0, fun = nxt ? nu : (T)0, fwn = nxt ? nw : (T)0;
        A = a * gu;
        B = a * gw + bd + c * fun;
        C = c * fwn;
        Dr = d - a * gy - c * fyn;
    }
    // parallel cyclic reduction over the lanes
#pragma unroll
    for (int st = 1; st < 32; st <<= 1) {
        T am = __shfl_up_sync(0xffffffffu, A, st), bm = __shfl_up_sync(0xffffffffu, B, st),
          cm = __shfl_up_sync(0xffffffffu, C, st), dm = __shfl_up_sync(0xffffffffu, Dr, st);
        T ap = __shfl_down_sync(0xffffffffu, A, st), bp = __shfl_down_sync(0xffffffffu, B, st),
          cq = __shfl_down_sync(0xffffffffu, C, st), dp = __shfl_down_sync(0xffffffffu, Dr, st);
        if (lane < st) {
            am = 0;
            bm = 1;
            cm = 0;
            dm = 0;
        }
        if (lane + st > 31) {
            ap = 0;
            bp = 1;
            cq = 0;
            dp = 0;
        }
        const T k1 = A / bm, k2 = C / bp;
        const T An = -am * k1, Cn = -cq * k2;
        const T Bn = B - cm * k1 - ap * k2, Dn = Dr - dm * k1 - dp * k2;
        A = An;
        B = Bn;
        C = Cn;
        Dr = Dn;
    }
    const T X = Dr / B;
    T Xm = __shfl_up_sync(0xffffffffu, X, 1);
    if (lane == 0) Xm = 0;
    // back substitution and the relaxation of the lane's rows
#pragma unroll
    for (int t = 0; t < kLineM; t++) {
        if (t < cnt) {
            const T xl = t < nl ? vy[t] + vu[t] * Xm + vw[t] * X : X;
            const long p = p0 + jo * (s + t + 1);
            const T xo = x[p];
            x[p] = xo + omega * (xl - xo);
        }
    }
}

// ---- residual + restriction ------------------------------------------------
// One coarse interior point per thread: the residuals of its 2x2x2 fine
// children are summed into the coarse right-hand side.
// residual of the 8 fine children of coarse point (i, j, k), summed.  With
// separable couplings the diagonal is their sum (the value whose
// reciprocal the smoother takes), so no division; Ix the offset type.
template <typename T, typename Ix = long>
__device__ __forceinline__ T rr_point(const BlkDev &f, int i, int j, int k, const T *__restrict__ E,
                                      const T *__restrict__ N, const T *__restrict__ R,
                                      const T *__restrict__ D, const T *__restrict__ x,
                                      const T *__restrict__ bb, const MfTab<T> &mf)
{
    const Ix jo = f.n[0], ko = (Ix)f.n[0] * f.n[1];
    const Ix p0 = (Ix)f.off3 + (2 * i - 3) + jo * (2 * j - 3) + ko * (2 * k - 3);
    T sum = 0;
#pragma unroll
    for (int dz = 0; dz < 2; dz++)
#pragma unroll
        for (int dy = 0; dy < 2; dy++)
#pragma unroll
            for (int dx = 0; dx < 2; dx++) {
                const Ix p = p0 + dx + jo * dy + ko * dz;
                T cf[6], dinv;
                if (mf.E2) {
                    const Ix ij = (Ix)f.off2 + (2 * i - 3 + dx) + jo * (2 * j - 3 + dy);
                    const Ix kk = (Ix)f.off1k + (2 * k - 3 + dz);
                    const T ez = mf.Ez[kk], nz = mf.Nz[kk], r2 = mf.R2[ij];
                    cf[0] = mf.E2[ij - 1] * ez;
                    cf[1] = mf.E2[ij] * ez;
                    cf[2] = mf.N2[ij - jo] * nz;
                    cf[3] = mf.N2[ij] * nz;
                    cf[4] = r2 * mf.Rz[kk - 1];
                    cf[5] = r2 * mf.Rz[kk];
                    const T ap = ((cf[0] + cf[1]) + (cf[2] + cf[3])) + (cf[4] + cf[5]);
                    const T ax = cf[0] * x[p - 1] + cf[1] * x[p + 1] + cf[2] * x[p - jo] + cf[3] * x[p + jo] +
                                 cf[4] * x[p - ko] + cf[5] * x[p + ko];
                    sum += bb[p] - x[p] * ap + ax;
                    continue;
                } else {
                    cf[0] = E[p - 1];
                    cf[1] = E[p];
                    cf[2] = N[p - jo];
                    cf[3] = N[p];
                    cf[4] = R[p - ko];
                    cf[5] = R[p];
                    dinv = D[p];
                }
                T ax = cf[0] * x[p - 1] + cf[1] * x[p + 1] + cf[2] * x[p - jo] + cf[3] * x[p + jo] +
                       cf[4] * x[p - ko] + cf[5] * x[p + ko];
                sum += bb[p] - x[p] / dinv + ax;
            }
    return sum;
}

// One coarse interior point per thread: the residuals of its 2x2x2 fine
// children are summed into the coarse right-hand side.  Thread (x, y) of
// CTA (bx, by, bz): coarse point i = 2 + 32 bx + x of row j = 2 +
// blockDim.y by + y of the coarse (block, plane) zmap[z0 + bz].
template <typename T, typename Ix>
__global__ void __launch_bounds__(256) k_resid_restrict(
    const BlkDev *__restrict__ bc_, const BlkDev *__restrict__ bf_, const T *__restrict__ E,
    const T *__restrict__ N, const T *__restrict__ R, const T *__restrict__ D,
    const T *__restrict__ x, const T *__restrict__ bb, T *__restrict__ bcoarse, MfTab<T> mf,
    const int2 *__restrict__ zmap, int z0)
{
    const int2 bk = zmap[z0 + blockIdx.z];
    const int bi = bk.x, k = bk.y;
    const BlkDev &c = bc_[bi];
    const int n0 = c.n[0], n1 = c.n[1];
    const int i = (int)(blockIdx.x * 32 + threadIdx.x) + 2, j = (int)(blockIdx.y * blockDim.y + threadIdx.y) + 2;
    if (k > c.n[2] - 1 || j > n1 - 1 || i > n0 - 1) return;
    const Ix pc = (Ix)c.off3 + (i - 1) + (Ix)n0 * (j - 1) + (Ix)n0 * n1 * (k - 1);
    pdl_wait();
    pdl_trigger();
    bcoarse[pc] = rr_point<T, Ix>(bf_[bi], i, j, k, E, N, R, D, x, bb, mf);
}

// ---- prolongation + correction --------------------------------------------
template <typename T>
__device__ __forceinline__ int clamp_c(int ic, int n, int lo_int, int hi_int)
{
    if (ic == 1 && !lo_int) return 2;
    if (ic == n && !hi_int) return n - 1;
    return ic;
}

// trilinear correction of fine interior point (i, j, k) at pf; Ix the
// offset type (int when every offset of the arrays is below 2^31)
template <typename T, typename Ix = long>
__device__ __forceinline__ void prolong_point(const BlkDev &c, const BlkDev &f, int bi, int i, int j,
                                              int k, Ix pf, const T *__restrict__ xc,
                                              T *__restrict__ xf, const PushDev *__restrict__ push)
{
    int ic = (i + 1) >> 1, a = (i + 1) & 1;
    int jc = (j + 1) >> 1, bq = (j + 1) & 1;
    int kc = (k + 1) >> 1, cq = (k + 1) & 1;
    // trilinear weights by the number h of axes on which the coarse point
    // is the far one: (3/4)^(3-h) (1/4)^h
    auto w = [](int h) -> T {
        return h == 0 ? (T)0.421875 : h == 1 ? (T)0.140625 : h == 2 ? (T)0.046875 : (T)0.015625;
    };
    bool iw = c.bc[0] == LES_BCT_INTERFACE_D, ie = c.bc[1] == LES_BCT_INTERFACE_D;
    bool js = c.bc[2] == LES_BCT_INTERFACE_D, jn = c.bc[3] == LES_BCT_INTERFACE_D;
    bool kl = c.bc[4] == LES_BCT_INTERFACE_D, kr = c.bc[5] == LES_BCT_INTERFACE_D;
    const Ix joc = c.n[0], koc = (Ix)c.n[0] * c.n[1], oc = (Ix)c.off3;
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
                cr += w(h) * xc[oc + (ii - 1) + joc * (jj - 1) + koc * (kk - 1)];
            }
    T v = xf[pf] + cr;
    xf[pf] = v;
    if (push && (i == 2 || i == f.n[0] - 1 || j == 2 || j == f.n[1] - 1 || k == 2 || k == f.n[2] - 1))
        push_ghosts(push + 6 * bi, f, i, j, k, v, xf);
}

// Thread (x, y) of CTA (bx, by, bz): the fine points 2c - 1 and 2c along
// each axis (c = 1 + 32 bx + x, 1 + blockDim.y by + y, and the coarse
// (block, plane) zmap[z0 + bz]; coarse c up to n - 1), i.e. the fine points whose
// coarse stencil is the 2 x 2 x 2 coarse points c..c+1 (clamped as
// prolong_point clamps).  The eight coarse values are loaded once for up to
// eight fine points; each fine point sums them in prolong_point's order.
template <typename T, typename Ix>
__global__ void __launch_bounds__(256) k_prolong8(const BlkDev *__restrict__ bc_, const BlkDev *__restrict__ bf_,
                                                  const T *__restrict__ xc, T *__restrict__ xf,
                                                  const PushDev *__restrict__ push, const int2 *__restrict__ zmap,
                                                  int z0)
{
    const int2 bk = zmap[z0 + blockIdx.z];
    const int bi = bk.x, cz = bk.y;
    const BlkDev &c = bc_[bi], &f = bf_[bi];
    const int cx = (int)(blockIdx.x * 32 + threadIdx.x) + 1, cy = (int)(blockIdx.y * blockDim.y + threadIdx.y) + 1;
    if (cx > c.n[0] - 1 || cy > c.n[1] - 1 || cz > c.n[2] - 1) return;
    const bool iw = c.bc[0] == LES_BCT_INTERFACE_D, ie = c.bc[1] == LES_BCT_INTERFACE_D;
    const bool js = c.bc[2] == LES_BCT_INTERFACE_D, jn = c.bc[3] == LES_BCT_INTERFACE_D;
    const bool kl = c.bc[4] == LES_BCT_INTERFACE_D, kr = c.bc[5] == LES_BCT_INTERFACE_D;
    const Ix joc = c.n[0], koc = (Ix)c.n[0] * c.n[1], oc = (Ix)c.off3;
    pdl_wait();
    pdl_trigger();
    T v[2][2][2];
#pragma unroll
    for (int sz = 0; sz < 2; sz++)
#pragma unroll
        for (int sy = 0; sy < 2; sy++)
#pragma unroll
            for (int sx = 0; sx < 2; sx++) {
                const int ii = clamp_c<T>(cx + sx, c.n[0], iw, ie);
                const int jj = clamp_c<T>(cy + sy, c.n[1], js, jn);
                const int kk = clamp_c<T>(cz + sz, c.n[2], kl, kr);
                v[sz][sy][sx] = xc[oc + (ii - 1) + joc * (jj - 1) + koc * (kk - 1)];
            }
    auto w = [](int h) -> T {
        return h == 0 ? (T)0.421875 : h == 1 ? (T)0.140625 : h == 2 ? (T)0.046875 : (T)0.015625;
    };
    const int n0 = f.n[0], n1 = f.n[1], n2 = f.n[2];
    const Ix jo = n0, ko = (Ix)n0 * n1, of = (Ix)f.off3;
#pragma unroll
    for (int dz = 0; dz < 2; dz++)
#pragma unroll
        for (int dy = 0; dy < 2; dy++)
#pragma unroll
            for (int dx = 0; dx < 2; dx++) {
                // fine point (2c - 1 + d): its coarse index is c and (i + 1) & 1 = d
                const int i = 2 * cx - 1 + dx, j = 2 * cy - 1 + dy, k = 2 * cz - 1 + dz;
                if (i < 2 || i > n0 - 1 || j < 2 || j > n1 - 1 || k < 2 || k > n2 - 1) continue;
                T cr = 0;
#pragma unroll
                for (int sz = 0; sz < 2; sz++)
#pragma unroll
                    for (int sy = 0; sy < 2; sy++)
#pragma unroll
                        for (int sx = 0; sx < 2; sx++)
                            cr += w((sx != dx) + (sy != dy) + (sz != dz)) * v[sz][sy][sx];
                const Ix pf = of + (i - 1) + jo * (j - 1) + ko * (k - 1);
                const T val = xf[pf] + cr;
                xf[pf] = val;
                if (push && (i == 2 || i == n0 - 1 || j == 2 || j == n1 - 1 || k == 2 || k == n2 - 1))
                    push_ghosts(push + 6 * bi, f, i, j, k, val, xf);
            }
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

// ---- the coarse tail of a V-cycle in one CTA --------------------------------
// Below a few tens of thousands of points a level's kernels are launch- and
// drain-bound (a few microseconds each for little work).  k_vtail runs the
// V-cycle from level l0 down to the coarsest level L and back -- smoothing,
// residual + restriction, coarsest-level mean removal and sweeps,
// prolongation -- as phases of one CTA separated by __syncthreads, the same
// operations in the same order as the per-level launches.
// per-block sums sb[] (block order) -> mean[b] = the interior mean over the
// connected component of block b; single thread, fixed order
__device__ __forceinline__ void comp_means_from_sums(const BlkDev *__restrict__ blk, int nb,
                                                     const double *sb, double *mean)
{
    double cs[kMaxBlk], cn[kMaxBlk];
    for (int q = 0; q < nb; q++) cs[q] = cn[q] = 0.;
    for (int b = 0; b < nb; b++) {
        const int cp = blk[b].comp;
        cs[cp] += sb[b];
        cn[cp] += (double)blk[b].ncell;
    }
    for (int b = 0; b < nb; b++) {
        const int cp = blk[b].comp;
        mean[b] = cn[cp] > 0. ? cs[cp] / cn[cp] : 0.;
    }
}

// per-block partial sums of k_interior_sum (gx per block) -> out[b], the
// interior mean over block b's component.  One CTA.
__global__ void k_comp_mean_final(const double *__restrict__ partial, int gx, int nb,
                                  const BlkDev *__restrict__ blk, double *__restrict__ out)
{
    __shared__ double sb[kMaxBlk];
    __shared__ double r[1];
    for (int b = 0; b < nb; b++) {
        double v[1] = {0.};
        for (int t = threadIdx.x; t < gx; t += blockDim.x) v[0] += partial[(long)b * gx + t];
        block_reduce_store<1>(v, r);
        __syncthreads();
        if (threadIdx.x == 0) sb[b] = r[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) comp_means_from_sums(blk, nb, sb, out);
}

// subtract from b, on every interior point, the mean of b over the point's
// component (all threads of the CTA take part)
template <typename T>
__device__ void remove_comp_means(const BlkDev *__restrict__ blk, int nb, T *__restrict__ bb)
{
    __shared__ double sb[kMaxBlk], mean[kMaxBlk];
    __shared__ double r[1];
    for (int ib = 0; ib < nb; ib++) {
        const BlkDev b = blk[ib];
        double v[1] = {0.};
        for (long q = threadIdx.x; q < b.ncell; q += blockDim.x) {
            int i, j, k;
            v[0] += (double)bb[decode_interior(b, q, i, j, k)];
        }
        block_reduce_store<1>(v, r);
        __syncthreads();
        if (threadIdx.x == 0) sb[ib] = r[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) comp_means_from_sums(blk, nb, sb, mean);
    __syncthreads();
    for (int ib = 0; ib < nb; ib++) {
        const BlkDev b = blk[ib];
        const T m = (T)mean[ib];
        for (long q = threadIdx.x; q < b.ncell; q += blockDim.x) {
            int i, j, k;
            bb[decode_interior(b, q, i, j, k)] -= m;
        }
    }
    __syncthreads();
}

template <typename T>
__device__ void tail_smooth(const VLev &L, int nb, int nsweep, T omega, const T *E, const T *N,
                            const T *R, const T *D, T *x, const T *bb, const MfTab<T> &mf)
{
    for (int sw = 0; sw < nsweep; sw++)
        for (int color = 0; color < 2; color++) {
            for (int bi = 0; bi < nb; bi++) {
                const BlkDev b = L.blk[bi];
                const unsigned nh = (unsigned)(b.n[0] - 1) >> 1;
                const unsigned tot = nh * (unsigned)(b.n[1] - 2) * (unsigned)(b.n[2] - 2);
                for (unsigned q = threadIdx.x; q < tot; q += blockDim.x) {
                    int i, j, k;
                    if (rb_decode(b, q, color, i, j, k))
                        rb_point(b, bi, i, j, k, omega, E, N, R, D, x, bb, L.rb_push ? L.push : nullptr, mf);
                }
            }
            __syncthreads();
            if (!L.rb_push && L.nface) {
                for (int fi = 0; fi < L.nface; fi++) {
                    const FaceDev f = L.face[fi];
                    const long nj = f.nj - 2, n = nj * (f.nk - 2);
                    for (long q = threadIdx.x; q < n; q += blockDim.x) {
                        long kk = q / nj + 1, jj = q - (kk - 1) * nj + 1;
                        x[f.gh + f.jo * jj + f.ko * kk] = x[f.ppk + f.pjo * jj + f.pko * kk];
                    }
                }
                __syncthreads();
            }
        }
}

// The bottom level solved exactly: b of its interior points gathered, x =
// A^-1 b by one dense product (cd.mt, built on the host from the level's
// couplings, ghosts folded into the columns of the points they mirror),
// written to the interior and pushed to the ghosts as a sweep would.
template <typename T>
__device__ void tail_direct(const VLev &L, int nb, const CoarseDirect<T> &cd, T *x, const T *bb)
{
    __shared__ T sb[kDirectMax];
    long g0 = 0;
    for (int bi = 0; bi < nb; bi++) {
        const BlkDev b = L.blk[bi];
        for (long q = threadIdx.x; q < b.ncell; q += blockDim.x) {
            int i, j, k;
            sb[g0 + q] = bb[decode_interior(b, q, i, j, k)];
        }
        g0 += b.ncell;
    }
    __syncthreads();
    g0 = 0;
    for (int bi = 0; bi < nb; bi++) {
        const BlkDev b = L.blk[bi];
        for (long q = threadIdx.x; q < b.ncell; q += blockDim.x) {
            const long g = g0 + q;
            T acc = 0;
            // the column reads are independent: many in flight (the inverse
            // comes from L2), the sum in the order of h
#pragma unroll 16
            for (int h = 0; h < cd.n; h++) acc += cd.mt[(long)h * cd.n + g] * sb[h];
            int i, j, k;
            const long p = decode_interior(b, q, i, j, k);
            x[p] = acc;
            if (L.rb_push) push_ghosts(L.push + 6 * bi, b, i, j, k, acc, x);
        }
        g0 += b.ncell;
    }
    __syncthreads();
    if (!L.rb_push && L.nface) {
        for (int fi = 0; fi < L.nface; fi++) {
            const FaceDev f = L.face[fi];
            const long nj = f.nj - 2, n = nj * (f.nk - 2);
            for (long q = threadIdx.x; q < n; q += blockDim.x) {
                long kk = q / nj + 1, jj = q - (kk - 1) * nj + 1;
                x[f.gh + f.jo * jj + f.ko * kk] = x[f.ppk + f.pjo * jj + f.pko * kk];
            }
        }
        __syncthreads();
    }
}

// The bottom level's operator for the host's dense inverse (one CTA): per
// interior point g (the order of tail_direct) its element index, the six
// couplings and 1/ap as the smoother forms them, and in `tag` (the level's
// elements) g at the point and at every ghost the sweeps fill from it (-1
// elsewhere).
template <typename T>
__global__ void __launch_bounds__(512) k_coarse_ops(const VLev *__restrict__ lvp, int lev, int nb, long base,
                                                    long len, const T *__restrict__ E, const T *__restrict__ N,
                                                    const T *__restrict__ R, const T *__restrict__ D, MfTab<T> mf,
                                                    float *__restrict__ tag, float *__restrict__ ops,
                                                    long *__restrict__ elem)
{
    const VLev L = lvp[lev];
    for (long q = threadIdx.x; q < len; q += blockDim.x) tag[q] = -1.f;
    __syncthreads();
    float *tg = tag - base;  // indexed by element
    long g0 = 0;
    for (int bi = 0; bi < nb; bi++) {
        const BlkDev b = L.blk[bi];
        const long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
        for (long q = threadIdx.x; q < b.ncell; q += blockDim.x) {
            int i, j, k;
            const long p = decode_interior(b, q, i, j, k), g = g0 + q;
            T c[6], dinv;
            if (mf.E2) {
                coefs_mf(b, mf, i, j, k, c, dinv);
            } else {
                c[0] = E[p - 1];
                c[1] = E[p];
                c[2] = N[p - jo];
                c[3] = N[p];
                c[4] = R[p - ko];
                c[5] = R[p];
                dinv = D[p];
            }
            for (int m = 0; m < 6; m++) ops[g * 7 + m] = (float)c[m];
            ops[g * 7 + 6] = (float)dinv;
            elem[g] = p;
            tg[p] = (float)g;
        }
        g0 += b.ncell;
    }
    __syncthreads();
    g0 = 0;
    for (int bi = 0; bi < nb; bi++) {
        const BlkDev b = L.blk[bi];
        for (long q = threadIdx.x; q < b.ncell; q += blockDim.x) {
            int i, j, k;
            decode_interior(b, q, i, j, k);
            if (L.rb_push) push_ghosts(L.push + 6 * bi, b, i, j, k, (float)(g0 + q), tg);
        }
        g0 += b.ncell;
    }
    __syncthreads();
    if (!L.rb_push)
        for (int fi = 0; fi < L.nface; fi++) {
            const FaceDev f = L.face[fi];
            const long nj = f.nj - 2, n = nj * (f.nk - 2);
            for (long q = threadIdx.x; q < n; q += blockDim.x) {
                long kk = q / nj + 1, jj = q - (kk - 1) * nj + 1;
                tg[f.gh + f.jo * jj + f.ko * kk] = tg[f.ppk + f.pjo * jj + f.pko * kk];
            }
            __syncthreads();
        }
}

// With `span` > 0 the tail's slice of the multigrid arrays (levels l0..L,
// elements [start, start + span)) is first copied into shared memory --
// x and b, and E, N, R, D unless the couplings are matrix-free -- and the
// same phases run there, each a __syncthreads apart instead of an L2
// round trip; x of the slice is copied back at the end (level l0's is
// what the prolongation to level l0-1 reads).
template <typename T>
__global__ void __launch_bounds__(512) k_vtail(const VLev *__restrict__ lv, int l0, int L, int nb,
                                                int pre, int crs, T omega, int singular,
                                                const T *__restrict__ E, const T *__restrict__ N,
                                                const T *__restrict__ R, const T *__restrict__ D,
                                                T *__restrict__ x, T *__restrict__ bb, MfTab<T> mf,
                                                long start, long span, CoarseDirect<T> cd)
{
    extern __shared__ __align__(16) unsigned char tail_smem[];
    T *const xg = x;
    pdl_wait();
    pdl_trigger();
    if (span > 0) {
        T *s = (T *)tail_smem;
        const int na = mf.E2 ? 2 : 6;
        const T *src[6] = {x, bb, E, N, R, D};
        for (int a = 0; a < na; a++)
            for (long q = threadIdx.x; q < span; q += blockDim.x) s[a * span + q] = src[a][start + q];
        __syncthreads();
        // the same indices (off3 of the levels) address the shared copies
        x = s - start;
        bb = s + span - start;
        if (!mf.E2) {
            E = s + 2 * span - start;
            N = s + 3 * span - start;
            R = s + 4 * span - start;
            D = s + 5 * span - start;
        }
    }
    for (int lev = l0; lev < L; lev++) {
        tail_smooth(lv[lev], nb, pre, omega, E, N, R, D, x, bb, mf);
        for (int bi = 0; bi < nb; bi++) {
            const BlkDev c = lv[lev + 1].blk[bi], f = lv[lev].blk[bi];
            for (long q = threadIdx.x; q < c.ncell; q += blockDim.x) {
                int i, j, k;
                long pc = decode_interior(c, q, i, j, k);
                bb[pc] = rr_point(f, i, j, k, E, N, R, D, x, bb, mf);
            }
        }
        __syncthreads();
    }
    if (singular) remove_comp_means<T>(lv[L].blk, nb, bb);
    if (cd.n > 0)
        tail_direct(lv[L], nb, cd, x, bb);
    else
        tail_smooth(lv[L], nb, L == 1 ? pre : crs, omega, E, N, R, D, x, bb, mf);
    for (int lev = L - 1; lev >= l0; lev--) {
        for (int bi = 0; bi < nb; bi++) {
            const BlkDev c = lv[lev + 1].blk[bi], f = lv[lev].blk[bi];
            for (long q = threadIdx.x; q < f.ncell; q += blockDim.x) {
                int i, j, k;
                long pf = decode_interior(f, q, i, j, k);
                prolong_point(c, f, bi, i, j, k, pf, x, x, lv[lev].push);
            }
        }
        __syncthreads();
        tail_smooth(lv[lev], nb, pre, omega, E, N, R, D, x, bb, mf);
    }
    if (span > 0) {
        __syncthreads();
        for (long q = threadIdx.x; q < span; q += blockDim.x) xg[start + q] = x[start + q];
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
    double *__restrict__ r64, double *__restrict__ partial)
{
    pdl_wait();
    pdl_trigger();
    const BlkDev b = blk[blockIdx.y];
    double v[2] = {0., 0.};
    const double s0 = shift ? shift[blockIdx.y] : 0.;
    // a warp per (j, k) row of the interior, grid-stride over rows
    const int ni = b.n[0] - 2;
    const unsigned nj = (unsigned)(b.n[1] - 2), nrow = nj * (unsigned)(b.n[2] - 2), wpb = blockDim.x >> 5;
    const long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    for (unsigned row = blockIdx.x * wpb + (threadIdx.x >> 5); row < nrow; row += gridDim.x * wpb) {
        const unsigned kq = row / nj;
        const long base = b.off3 + 1 + jo * (long)(row - kq * nj + 1) + ko * (long)(kq + 1);
        for (int iq = threadIdx.x & 31; iq < ni; iq += 32) {
            const long p = base + iq;
            const double bp = bb[p] - s0;
            double r = bp - P[p] * x[p] + E[p - 1] * x[p - 1] + E[p] * x[p + 1] + N[p - jo] * x[p - jo] +
                       N[p] * x[p + jo] + R[p - ko] * x[p - ko] + R[p] * x[p + ko];
            rT[p] = (T)r;
            if (r64) r64[p] = r;
            v[0] += r * r;
            v[1] += bp * bp;
        }
    }
    block_reduce_store<2>(v, partial + 2 * (blockIdx.y * (long)gridDim.x + blockIdx.x));
}

__global__ void k_sum2_final(const double *__restrict__ partial, long nparts, double *__restrict__ out)
{
    pdl_wait();
    pdl_trigger();
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

// Coarsest level of a singular (pure Neumann / periodic) operator: remove
// the mean of the right-hand side over each component's interior points so
// the coarse problem is compatible and its smoothing cannot drift along the
// constant null vectors.  One CTA; the level has a few hundred points at most.
template <typename T>
__global__ void k_coarse_mean(const BlkDev *__restrict__ blk, int nb, T *__restrict__ bb)
{
    remove_comp_means<T>(blk, nb, bb);
}

// p += e on the interior of level 1.  Thread (x, y) of CTA (bx, by, bz):
// point i = 2 + 32 bx + x of row j = 2 + blockDim.y by + y of the (block,
// plane) zmap[z0 + bz].
template <typename T, typename Ix>
__global__ void k_update(const BlkDev *__restrict__ blk, double *__restrict__ p,
                         const T *__restrict__ e, const PushDev *__restrict__ push, const int2 *__restrict__ zmap,
                         int z0)
{
    const int2 bk = zmap[z0 + blockIdx.z];
    const int bi = bk.x, k = bk.y;
    const int n0 = blk[bi].n[0], n1 = blk[bi].n[1], n2 = blk[bi].n[2];
    const int i = (int)(blockIdx.x * 32 + threadIdx.x) + 2, j = (int)(blockIdx.y * blockDim.y + threadIdx.y) + 2;
    if (k > n2 - 1 || j > n1 - 1 || i > n0 - 1) return;
    const Ix pp = (Ix)blk[bi].off3 + (i - 1) + (Ix)n0 * (j - 1) + (Ix)n0 * n1 * (k - 1);
    double v = p[pp] + (double)e[pp];
    p[pp] = v;
    if (push && (i == 2 || i == n0 - 1 || j == 2 || j == n1 - 1 || k == 2 || k == n2 - 1))
        push_ghosts(push + 6 * bi, blk[bi], i, j, k, v, p);
}

// ---- flexible conjugate gradients around the V-cycle ----------------------
// FCG(1): with z = V(r) the cycle's correction for the residual r,
//   beta = (z.q) / (p.q),  p <- z - beta p,  q <- A z - beta q   (q = A p)
//   alpha = (p.r) / (p.q), x <- x + alpha p,  r <- r - alpha q
// The scalars stay on the device: sc[0] = z.q, sc[2] = p.q, sc[3] = p.r
// (sc[2] = 0 restarts with beta = 0).  Interior points of level 1; the
// reductions are per-CTA partials summed by k_sum2_final.

// partial sums of z.q (and z.r)
template <typename T>
__global__ void __launch_bounds__(256) k_fcg_dot(const BlkDev *__restrict__ blk, const T *__restrict__ z,
                                                 const double *__restrict__ q, const double *__restrict__ r,
                                                 double *__restrict__ partial)
{
    const BlkDev b = blk[blockIdx.y];
    double v[2] = {0., 0.};
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < b.ncell; t += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        long p = decode_interior(b, t, i, j, k);
        const double zp = (double)z[p];
        v[0] += zp * q[p];
        v[1] += zp * r[p];
    }
    block_reduce_store<2>(v, partial + 2 * (blockIdx.y * (long)gridDim.x + blockIdx.x));
}

// new direction p and q = A p (FP64 coefficients, z's ghosts current);
// partial sums of p.q and p.r
template <typename T>
__global__ void __launch_bounds__(256) k_fcg_dir(
    const BlkDev *__restrict__ blk, const double *__restrict__ E, const double *__restrict__ N,
    const double *__restrict__ R, const double *__restrict__ P, const T *__restrict__ z,
    double *__restrict__ pd, double *__restrict__ q, const double *__restrict__ r,
    const double *__restrict__ sc, double *__restrict__ partial)
{
    const BlkDev b = blk[blockIdx.y];
    const double pq = sc[2];
    const double beta = pq != 0. ? sc[0] / pq : 0.;
    double v[2] = {0., 0.};
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < b.ncell; t += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        long p = decode_interior(b, t, i, j, k);
        long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
        double az = P[p] * (double)z[p] - E[p - 1] * (double)z[p - 1] - E[p] * (double)z[p + 1] -
                    N[p - jo] * (double)z[p - jo] - N[p] * (double)z[p + jo] -
                    R[p - ko] * (double)z[p - ko] - R[p] * (double)z[p + ko];
        double pn = (double)z[p] - beta * pd[p];
        double qn = az - beta * q[p];
        pd[p] = pn;
        q[p] = qn;
        v[0] += pn * qn;
        v[1] += pn * r[p];
    }
    block_reduce_store<2>(v, partial + 2 * (blockIdx.y * (long)gridDim.x + blockIdx.x));
}

// x += alpha p (with the ghost mirrors), r -= alpha q, rT = r; partial r.r
template <typename T>
__global__ void __launch_bounds__(256) k_fcg_step(const BlkDev *__restrict__ blk, double *__restrict__ x,
                                                  const double *__restrict__ pd, const double *__restrict__ q,
                                                  double *__restrict__ r, T *__restrict__ rT,
                                                  const double *__restrict__ sc, const PushDev *__restrict__ push,
                                                  double *__restrict__ partial)
{
    const BlkDev b = blk[blockIdx.y];
    const double pq = sc[2];
    const double alpha = pq != 0. ? sc[3] / pq : 0.;
    double v[2] = {0., 0.};
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < b.ncell; t += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        long p = decode_interior(b, t, i, j, k);
        double xn = x[p] + alpha * pd[p];
        x[p] = xn;
        if (push) push_ghosts(push + 6 * blockIdx.y, b, i, j, k, xn, x);
        double rn = r[p] - alpha * q[p];
        r[p] = rn;
        rT[p] = (T)rn;
        v[0] += rn * rn;
    }
    block_reduce_store<2>(v, partial + 2 * (blockIdx.y * (long)gridDim.x + blockIdx.x));
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

// maxn: the most points (ghosts included) of a block along i, j, k;
// threads per CTA 128, 256 or 512 (4, 8 or 16 rows of 32); wide: 64-bit
// offsets (the multigrid arrays hold 2^31 points or more)
template <typename T>
void launch_rb(const BlkDev *blk, int nb, const int maxn[3], int color, double omega, const T *E,
               const T *N, const T *R, const T *D, T *x, const T *b, const PushDev *push,
               const MfTab<T> &mf, int threads, bool wide, const LevGeo *geo, ZMap zm, cudaStream_t st)
{
    const int rows = (threads == 128 || threads == 512) ? threads / 32 : 8;
    if (geo && !wide && zm.n <= 65535) {
        const dim3 grid(nb_((maxn[0] - 1) / 2, 32), nb_(maxn[1] - 2, rows), (unsigned)zm.n);
        const dim3 cta(32, rows);
        const T om = (T)omega;
#define LES_RB_GEO(MF, ONE, PUSH)                                                                            \
    launch_pdl(k_rb_geo<T, MF, ONE, PUSH>, grid, cta, 0, st, *geo, color, om, E, N, R, D, x, b, mf, zm.map)
        const bool one = geo->nb == 1, pu = push != nullptr;
        if (mf.E2) {
            if (one) { if (pu) LES_RB_GEO(true, true, true); else LES_RB_GEO(true, true, false); }
            else { if (pu) LES_RB_GEO(true, false, true); else LES_RB_GEO(true, false, false); }
        } else {
            if (one) { if (pu) LES_RB_GEO(false, true, true); else LES_RB_GEO(false, true, false); }
            else { if (pu) LES_RB_GEO(false, false, true); else LES_RB_GEO(false, false, false); }
        }
#undef LES_RB_GEO
        count_launch(1);
        return;
    }
    // gridDim.z <= 65535: the (block, plane) pairs in groups
    for (int z0 = 0; z0 < zm.n; z0 += 65535) {
        const dim3 grid(nb_((maxn[0] - 1) / 2, 32), nb_(maxn[1] - 2, rows), (unsigned)std::min(65535, zm.n - z0));
        const dim3 cta(32, rows);
        const T om = (T)omega;
        if (!wide && mf.E2)
            launch_pdl(k_rb<T, true, int>, grid, cta, 0, st, blk, color, om, E, N, R, D, x, b, push, mf, zm.map, z0);
        else if (!wide)
            launch_pdl(k_rb<T, false, int>, grid, cta, 0, st, blk, color, om, E, N, R, D, x, b, push, mf, zm.map, z0);
        else if (mf.E2)
            launch_pdl(k_rb<T, true, long>, grid, cta, 0, st, blk, color, om, E, N, R, D, x, b, push, mf, zm.map, z0);
        else
            launch_pdl(k_rb<T, false, long>, grid, cta, 0, st, blk, color, om, E, N, R, D, x, b, push, mf, zm.map,
                       z0);
        count_launch(1);
    }
}

template <typename T> __global__ void k_copy_range(const T *__restrict__ src, T *__restrict__ dst, long n)
{
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        dst[q] = src[q];
}

template <typename T> void launch_copy_range(const T *src, T *dst, long n, cudaStream_t st)
{
    unsigned g = nb_(n, 256);
    k_copy_range<T><<<g > 2432 ? 2432 : g, 256, 0, st>>>(src, dst, n);
    count_launch(1);
}

template <typename T>
void launch_rb_tile(const BlkDev *blk, const int n[3], double omega, const T *xin, T *xout, const T *b,
                    const PushDev *push, const MfTab<T> &mf, cudaStream_t st)
{
    const int ntile = ((n[0] - 2 + kTI - 1) / kTI) * ((n[1] - 2 + kTJ - 1) / kTJ) * ((n[2] - 2 + kTK - 1) / kTK);
    k_rb_tile<T><<<ntile, 256, kRbTileSmem<T>, st>>>(blk, (T)omega, xin, xout, b, push, mf);
    count_launch(1);
}

template <typename T>
void launch_yline(const BlkDev *blk, int nb, long maxik_half, int color, double omega, const T *E, const T *N,
                  const T *R, const T *D, T *x, const T *b, const MfTab<T> &mf, T *cp, T *dp, int maxnj,
                  cudaStream_t st)
{
    // a warp per line (4 per CTA of 128 threads) where the lines are few:
    // with tens of thousands of lines a thread per line already fills the
    // GPU and does less work in all (measured on the 512x384x256 channel's
    // level 1, 65536 lines a colour: the warps were slower)
    if (maxnj <= 32 * kLineM && maxik_half * nb <= 8192)
        k_yline_warp<T><<<dim3(nb_(maxik_half, 4), nb), 128, 0, st>>>(blk, color, (T)omega, E, N, R, D, x, b, mf);
    else
        k_yline<T><<<dim3(nb_(maxik_half, 128), nb), 128, 0, st>>>(blk, color, (T)omega, E, N, R, D, x, b, mf, cp,
                                                                   dp);
    count_launch(1);
}

template <typename T>
void launch_resid_restrict(const BlkDev *bc, const BlkDev *bf, int nb, const int maxn_c[3], const T *E,
                           const T *N, const T *R, const T *D, const T *x, const T *b, T *bcoarse,
                           const MfTab<T> &mf, bool wide, ZMap zm_c, cudaStream_t st)
{
    for (int z0 = 0; z0 < zm_c.n; z0 += 65535) {
        const dim3 grid(nb_(maxn_c[0] - 2, 32), nb_(maxn_c[1] - 2, 8), (unsigned)std::min(65535, zm_c.n - z0));
        if (wide)
            launch_pdl(k_resid_restrict<T, long>, grid, dim3(32, 8), 0, st, bc, bf, E, N, R, D, x, b, bcoarse, mf,
                       zm_c.map, z0);
        else
            launch_pdl(k_resid_restrict<T, int>, grid, dim3(32, 8), 0, st, bc, bf, E, N, R, D, x, b, bcoarse, mf,
                       zm_c.map, z0);
        count_launch(1);
    }
}

template <typename T>
void launch_prolong_fast(const BlkDev *bc, const BlkDev *bf, int nb, const int maxn_f[3], const T *xc,
                         T *xf, const PushDev *push, bool wide, ZMap zm_c, cudaStream_t st)
{
    // a thread per coarse c = 1 .. n_coarse - 1 along each axis: the fine
    // level has n_fine = 2 n_coarse - 2 points per axis, ghosts included;
    // zm_c: the coarse (block, plane) pairs, planes 1 .. n_coarse - 1
    const int mc[2] = {maxn_f[0] / 2 + 1, maxn_f[1] / 2 + 1};
    for (int z0 = 0; z0 < zm_c.n; z0 += 65535) {
        const dim3 grid(nb_(mc[0] - 1, 32), nb_(mc[1] - 1, 8), (unsigned)std::min(65535, zm_c.n - z0));
        if (wide)
            launch_pdl(k_prolong8<T, long>, grid, dim3(32, 8), 0, st, bc, bf, xc, xf, push, zm_c.map, z0);
        else
            launch_pdl(k_prolong8<T, int>, grid, dim3(32, 8), 0, st, bc, bf, xc, xf, push, zm_c.map, z0);
        count_launch(1);
    }
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
void launch_resid_outer(const BlkDev *blk, int nb, long maxrow, const double *E, const double *N,
                        const double *R, const double *P, const double *x, const double *b,
                        const double *shift, T *rT, double *r64, double *partial, double *out2,
                        cudaStream_t st)
{
    // grid-stride over rows: a few CTAs per SM (so that the final sum reads
    // few partials), every warp the same number of rows
    const long cap = (1216 + nb - 1) / nb, per = (maxrow + 8 * cap - 1) / (8 * cap);
    const unsigned gx = (unsigned)std::max(1L, (maxrow + 8 * per - 1) / (8 * per));
    launch_pdl(k_resid_outer<T>, dim3(gx, nb), dim3(256), 0, st, blk, E, N, R, P, x, b, shift, rT, r64, partial);
    launch_pdl(k_sum2_final, dim3(1), dim3(256), 0, st, partial, (long)gx * nb, out2);
    count_launch(2);
}

static unsigned reduce_grid(long maxcell, int nb)
{
    unsigned gx = nb_(maxcell, 256);
    unsigned cap = (unsigned)((1216 + nb - 1) / nb);
    return gx > cap ? cap : gx;
}

template <typename T>
void launch_fcg(const BlkDev *blk, int nb, long maxcell, const double *E, const double *N, const double *R,
                const double *P, const T *z, double *x, double *pd, double *q, double *r, T *rT,
                const PushDev *push, double *partial, double *sc, double *out_rr, cudaStream_t st)
{
    unsigned gx = reduce_grid(maxcell, nb);
    long np = (long)gx * nb;
    k_fcg_dot<T><<<dim3(gx, nb), 256, 0, st>>>(blk, z, q, r, partial);
    launch_pdl(k_sum2_final, dim3(1), dim3(256), 0, st, partial, np, sc);
    k_fcg_dir<T><<<dim3(gx, nb), 256, 0, st>>>(blk, E, N, R, P, z, pd, q, r, sc, partial);
    launch_pdl(k_sum2_final, dim3(1), dim3(256), 0, st, partial, np, sc + 2);
    k_fcg_step<T><<<dim3(gx, nb), 256, 0, st>>>(blk, x, pd, q, r, rT, sc, push, partial);
    launch_pdl(k_sum2_final, dim3(1), dim3(256), 0, st, partial, np, out_rr);
    count_launch(6);
}

void launch_interior_mean(const BlkDev *blk, int nb, long maxcell, const double *b, double *partial,
                          double *out, cudaStream_t st)
{
    unsigned gx = nb_(maxcell, 256);
    unsigned cap = (unsigned)((1216 + nb - 1) / nb);
    if (gx > cap) gx = cap;
    k_interior_sum<<<dim3(gx, nb), 256, 0, st>>>(blk, b, partial);
    k_comp_mean_final<<<1, 256, 0, st>>>(partial, (int)gx, nb, blk, out);
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
        launch_pdl(k_recip, dim3(gx, m), dim3(256), 0, st, J, n);
        count_launch(1);
    }
}

void launch_to_f32(const double *const *src, float *const *dst, int ntab, long n, cudaStream_t st)
{
    F32Job J;
    for (int b0 = 0; b0 < ntab; b0 += 24) {
        int m = ntab - b0 < 24 ? ntab - b0 : 24;
        for (int t = 0; t < m; t++) {
            J.src[t] = src[b0 + t];
            J.dst[t] = dst[b0 + t];
        }
        unsigned gx = nb_(n, 256);
        if (gx > 256) gx = 256;
        launch_pdl(k_to_f32, dim3(gx, m), dim3(256), 0, st, J, n);
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
void launch_update(const BlkDev *blk, int nb, const int maxn[3], double *p, const T *e, const PushDev *push,
                   bool wide, ZMap zm, cudaStream_t st)
{
    for (int z0 = 0; z0 < zm.n; z0 += 65535) {
        const dim3 grid(nb_(maxn[0] - 2, 32), nb_(maxn[1] - 2, 8), (unsigned)std::min(65535, zm.n - z0));
        if (wide)
            k_update<T, long><<<grid, dim3(32, 8), 0, st>>>(blk, p, e, push, zm.map, z0);
        else
            k_update<T, int><<<grid, dim3(32, 8), 0, st>>>(blk, p, e, push, zm.map, z0);
        count_launch(1);
    }
}

template <typename T>
void launch_mf_tables(const BlkDev *blk, int nb, long maxcell, long max2d, int maxn2, const T *E,
                      const T *N, const T *R, const T *D, const MfTab<T> &t, double tol, int *bad,
                      cudaStream_t st)
{
    long n = max2d > maxn2 ? max2d : maxn2;
    k_mf_extract<T><<<dim3(nb_(n, 256), nb), 256, 0, st>>>(blk, E, N, R, t, bad);
    k_mf_check<T><<<dim3(nb_(maxcell, 256), nb), 256, 0, st>>>(blk, E, N, R, D, t, (T)tol, bad);
    count_launch(2);
}

template <typename T>
void launch_vtail(const VLev *lv, int l0, int L, int nb, int pre, int crs, double omega, int singular,
                  const T *E, const T *N, const T *R, const T *D, T *x, T *b, const MfTab<T> &mf,
                  long start, long span, const CoarseDirect<T> &cd, cudaStream_t st)
{
    // the slice in shared memory where it fits (kVtailSmem, the limit
    // prepare_vtail set)
    const size_t smem = span > 0 ? (size_t)span * (mf.E2 ? 2 : 6) * sizeof(T) : 0;
    const T om = (T)omega;
    if (smem == 0 || smem > kVtailSmem)
        launch_pdl(k_vtail<T>, dim3(1), dim3(512), 0, st, lv, l0, L, nb, pre, crs, om, singular, E, N, R, D, x, b, mf,
                   0L, 0L, cd);
    else
        launch_pdl(k_vtail<T>, dim3(1), dim3(512), smem, st, lv, l0, L, nb, pre, crs, om, singular, E, N, R, D, x, b,
                   mf, start, span, cd);
    count_launch(1);
}

template <typename T>
void launch_coarse_ops(const VLev *lv, int lev, int nb, long base, long len, const T *E, const T *N, const T *R,
                       const T *D, const MfTab<T> &mf, float *tag, float *ops, long *elem, cudaStream_t st)
{
    k_coarse_ops<T><<<1, 512, 0, st>>>(lv, lev, nb, base, len, E, N, R, D, mf, tag, ops, elem);
    count_launch(1);
}

// the tail kernels' shared-memory limit, set once per context (outside any
// stream capture); false where the device refuses it (the tail then runs in
// global memory... only if the caller checks: launch_vtail uses the limit)
bool prepare_vtail()
{
    bool ok = cudaFuncSetAttribute(k_vtail<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kVtailSmem) ==
                  cudaSuccess &&
              cudaFuncSetAttribute(k_vtail<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kVtailSmem) ==
                  cudaSuccess;
    if (!ok) cudaGetLastError();
    return ok;
}

// the shared-memory red-black tiles' shared memory limit, once per context
bool prepare_rb_tile()
{
    // the largest shared-memory carveout, so that several tiles share an SM
    const bool ok = cudaFuncSetAttribute(k_rb_tile<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kRbTileSmem<float>) == cudaSuccess &&
                    cudaFuncSetAttribute(k_rb_tile<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kRbTileSmem<double>) == cudaSuccess &&
                    cudaFuncSetAttribute(k_rb_tile<float>, cudaFuncAttributePreferredSharedMemoryCarveout, 100) ==
                        cudaSuccess &&
                    cudaFuncSetAttribute(k_rb_tile<double>, cudaFuncAttributePreferredSharedMemoryCarveout, 100) ==
                        cudaSuccess;
    if (!ok) cudaGetLastError();
    return ok;
}

#define INST(T)                                                                                    \
    template int launch_conv_coef<T>(const BlkDev *, int, long, const double *const *, T *, T *,   \
                                     T *, T *, double *, double *, double *, double *, int *,     \
                                     cudaStream_t);                                                \
    template void launch_rb<T>(const BlkDev *, int, const int *, int, double, const T *, const T *, \
                               const T *, const T *, T *, const T *, const PushDev *,             \
                               const MfTab<T> &, int, bool, const LevGeo *, ZMap, cudaStream_t);  \
    template void launch_yline<T>(const BlkDev *, int, long, int, double, const T *, const T *,   \
                                  const T *, const T *, T *, const T *, const MfTab<T> &, T *, T *, \
                                  int, cudaStream_t);                                             \
    template void launch_resid_restrict<T>(const BlkDev *, const BlkDev *, int, const int *, const T *, \
                                           const T *, const T *, const T *, const T *, const T *, \
                                           T *, const MfTab<T> &, bool, ZMap, cudaStream_t);      \
    template void launch_vtail<T>(const VLev *, int, int, int, int, int, double, int, const T *,   \
                                  const T *, const T *, const T *, T *, T *, const MfTab<T> &,    \
                                  long, long, const CoarseDirect<T> &, cudaStream_t);             \
    template void launch_copy_range<T>(const T *, T *, long, cudaStream_t);                        \
    template void launch_rb_tile<T>(const BlkDev *, const int *, double, const T *, T *, const T *, \
                                    const PushDev *, const MfTab<T> &, cudaStream_t);             \
    template void launch_coarse_ops<T>(const VLev *, int, int, long, long, const T *, const T *,  \
                                       const T *, const T *, const MfTab<T> &, float *, float *,  \
                                       long *, cudaStream_t);                                     \
    template void launch_mf_tables<T>(const BlkDev *, int, long, long, int, const T *, const T *, \
                                      const T *, const T *, const MfTab<T> &, double, int *,      \
                                      cudaStream_t);                                              \
    template void launch_prolong_fast<T>(const BlkDev *, const BlkDev *, int, const int *, const T *, \
                                         T *, const PushDev *, bool, ZMap, cudaStream_t);         \
    template void launch_halo_fast<T>(const FaceDev *, int, long, T *, cudaStream_t);             \
    template void launch_resid_outer<T>(const BlkDev *, int, long, const double *,                \
                                        const double *, const double *, const double *,           \
                                        const double *, const double *, const double *, T *,      \
                                        double *, double *, double *, cudaStream_t);              \
    template void launch_fcg<T>(const BlkDev *, int, long, const double *, const double *,        \
                                const double *, const double *, const T *, double *, double *,   \
                                double *, double *, T *, const PushDev *, double *, double *,    \
                                double *, cudaStream_t);                                         \
    template void launch_update<T>(const BlkDev *, int, const int *, double *, const T *, const PushDev *, bool, \
                                   ZMap, cudaStream_t);                                          \
    template void launch_coarse_mean<T>(const BlkDev *, int, T *, cudaStream_t);
INST(float)
INST(double)
#undef INST

} // namespace les
