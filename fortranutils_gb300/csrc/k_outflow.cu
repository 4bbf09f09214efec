// k_outflow.cu -- convective outflow and fixed inflow sides:
//   conv_exitbc1_block / conv_exitbc2_block (code/conv_exitbc1_block.F,
//   conv_exitbc2_block.F), conv_exitbc_scale (conv_exitbc_scale.F),
//   mass_flux (mass_flux.F), mass_change_block (mass_change_block.F),
//   fixed_inlet (fixed_inlet.F).
// Compiled with -fmad=false: the per-point updates round as the Fortran
// does.  The plane and volume sums are CTA tree reductions (fixed order),
// equal to the reference's sequential sums up to rounding.
#include "k_common.cuh"
#include "kernels.h"

// mass_flux over one side's exit plane (code/mass_flux.F:48-99), one CTA per
// side; out[3 q + 0..2] = area, rho-weighted area, mass flux.  which: 0 the
// fixed sides, 1 the convective ones, 2 both; iva 0 = each side's own axis,
// else zero unless the side's axis is iva's (mass_flux.F:40)
__global__ void k_side_flux(const SideJob *__restrict__ jobs, int iva, int which, const double *__restrict__ u,
                            const double *__restrict__ v, const double *__restrict__ w,
                            const double *__restrict__ rho, const double *__restrict__ rdju,
                            const double *__restrict__ rdiv, const double *__restrict__ didjp,
                            const double *__restrict__ dkp, double *__restrict__ out)
{
    const SideJob J = jobs[blockIdx.x];
    double v3[3] = {0., 0., 0.};
    const bool active = (which == 2 || J.conv == which) && (iva == 0 || J.d1 == iva);
    if (active) {
        const int *se = J.bnd[J.d1];
        const long jo = J.n[0], ko = (long)J.n[0] * J.n[1];
        const int plane = J.plane;
        if (J.d1 == 1) {
            const int nj = se[3] - se[2] + 1, nk = se[5] - se[4] + 1;
            for (int q = threadIdx.x; q < nj * nk; q += blockDim.x) {
                const int j = se[2] + q % nj, k = se[4] + q / nj;
                const long ijk = J.off3 + (plane - 1) + jo * (j - 1) + ko * (k - 1);
                const double areaf = rdju[J.off2 + (plane - 1) + jo * (j - 1)] * dkp[J.off1k + k - 1];
                const double r = 0.5 * (rho[ijk] + rho[ijk - 1]);
                v3[0] += areaf;
                v3[1] += r * areaf;
                v3[2] += r * u[ijk] * areaf;
            }
        } else if (J.d1 == 2) {
            const int ni = se[1] - se[0] + 1, nk = se[5] - se[4] + 1;
            for (int q = threadIdx.x; q < ni * nk; q += blockDim.x) {
                const int i = se[0] + q % ni, k = se[4] + q / ni;
                const long ijk = J.off3 + (i - 1) + jo * (plane - 1) + ko * (k - 1);
                const double areaf = rdiv[J.off2 + (i - 1) + jo * (plane - 1)] * dkp[J.off1k + k - 1];
                const double r = 0.5 * (rho[ijk] + rho[ijk - jo]);
                v3[0] += areaf;
                v3[1] += r * areaf;
                v3[2] += r * v[ijk] * areaf;
            }
        } else {
            const int ni = se[1] - se[0] + 1, nj = se[3] - se[2] + 1;
            for (int q = threadIdx.x; q < ni * nj; q += blockDim.x) {
                const int i = se[0] + q % ni, j = se[2] + q / ni;
                const long ijk = J.off3 + (i - 1) + jo * (j - 1) + ko * (plane - 1);
                const double areaf = didjp[J.off2 + (i - 1) + jo * (j - 1)];
                const double r = 0.5 * (rho[ijk] + rho[ijk - ko]);
                v3[0] += areaf;
                v3[1] += r * areaf;
                v3[2] += r * w[ijk] * areaf;
            }
        }
    }
    __shared__ double tot[3];
    block_reduce_store<3>(v3, tot);
    __syncthreads();
    if (threadIdx.x == 0) {
        out[3 * blockIdx.x + 0] = tot[0];
        out[3 * blockIdx.x + 1] = tot[1];
        out[3 * blockIdx.x + 2] = tot[2];
    }
}

// the side sums into the SAVEd totals, in (block, side) order:
// mode 0: per-side outflow totals (ttl, arho) of the convective sides;
// mode 1: mflux_in += fixed sides; mode 2: mflux_out += convective sides;
// mode 3: both sums zeroed first (iva = u)
__global__ void k_side_combine(const SideJob *__restrict__ jobs, int njobs, const double *__restrict__ out,
                               int mode, double *__restrict__ ex)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (mode == 0) {
        for (int s = 1; s <= 6; s++) ex[EX_TTL + s] = ex[EX_ARHO + s] = 0.;
        for (int q = 0; q < njobs; q++)
            if (jobs[q].conv) {
                ex[EX_TTL + jobs[q].side] = ex[EX_TTL + jobs[q].side] + out[3 * q + 2];
                ex[EX_ARHO + jobs[q].side] = ex[EX_ARHO + jobs[q].side] + out[3 * q + 1];
            }
        return;
    }
    if (mode == 3) {
        ex[EX_IN] = 0.;
        ex[EX_OUT] = 0.;
        return;
    }
    for (int q = 0; q < njobs; q++) {
        if (mode == 1 && !jobs[q].conv) ex[EX_IN] = ex[EX_IN] + out[3 * q + 2];
        if (mode == 2 && jobs[q].conv) ex[EX_OUT] = ex[EX_OUT] + out[3 * q + 2];
    }
}

// conv_exitbc1_block (task 1) / conv_exitbc2_block (task 2) for one
// variable on every convective side, one CTA per side.  dm, rm, km: the
// metric arguments conv_exitbc.F passes for (d1, iva), chosen by the host
// per axis: dm[d1], rm[d1], km[d1].
__global__ void k_exit_update(const SideJob *__restrict__ jobs, int task, int iva, ExitMetrics M,
                              double *__restrict__ u, double *__restrict__ u_int,
                              const double *__restrict__ rho, const double *__restrict__ rhonp1,
                              double *__restrict__ hn, double dtime, const double *__restrict__ ex)
{
    const SideJob J = jobs[blockIdx.x];
    if (!J.conv) return;
    const int d1 = J.d1;
    const double *dm = M.dm[d1], *rm = M.rm[d1], *km = M.km[d1];
    const int *r = J.bnd[iva];
    const long n0 = J.n[0], ld = (long)J.n[0] * J.n[1];
    const double uave = ex[EX_TTL + J.side] / ex[EX_ARHO + J.side];
    const double const1 = 1.5 * dtime, const2 = 0.5 * dtime;
    const bool low = (J.side % 2) == 1;
    // routine roles: a = the exit axis, (b, c) = the loop axes
    long sa, sb, sc;
    int b0, b1, c0, c1, pa, pa1;
    if (d1 == 1) {
        sa = 1; sb = n0; sc = ld;
        b0 = r[2]; b1 = r[3]; c0 = r[4]; c1 = r[5];
        pa = low ? r[0] - 1 : r[1] + 1; pa1 = low ? r[0] : r[1];
    } else if (d1 == 2) {
        sa = n0; sb = 1; sc = ld;
        b0 = r[0]; b1 = r[1]; c0 = r[4]; c1 = r[5];
        pa = low ? r[2] - 1 : r[3] + 1; pa1 = low ? r[2] : r[3];
    } else {
        sa = ld; sb = 1; sc = n0;
        b0 = r[0]; b1 = r[1]; c0 = r[2]; c1 = r[3];
        pa = low ? r[4] - 1 : r[5] + 1; pa1 = low ? r[4] : r[5];
    }
    const long off = low ? -sa : sa, off2 = low ? 0 : sa;
    const double uave1 = low ? -uave : uave;
    const int nb = b1 - b0 + 1, nc = c1 - c0 + 1;
    for (int q = threadIdx.x; q < nb * nc; q += blockDim.x) {
        const int bb = b0 + q % nb, cc = c0 + q / nb;
        const long ijk = J.off3 + sa * (pa - 1) + sb * (bb - 1) + sc * (cc - 1);
        if (task == 2) {
            u[ijk] = u_int[ijk];
            continue;
        }
        const long ijk2 = ijk - off2;
        double dx;
        if (d1 == 1) {
            dx = dm[J.off2 + (pa1 - 1) + n0 * (bb - 1)];
        } else if (d1 == 2) {
            dx = dm[J.off2 + (bb - 1) + n0 * (pa1 - 1)];
        } else {
            dx = rm[J.off2 + (bb - 1) + n0 * (cc - 1)] * km[J.off1k + pa1 - 1];
        }
        const double rho1 = 0.5 * (rho[ijk2] + rho[ijk2 + off]);
        const double rho2 = 0.5 * (rho[ijk2] + rho[ijk2 - off]);
        const double h = uave1 * (rho1 * u[ijk] - rho2 * u[ijk - off]) / dx;
        const double rhonp1_1 = 0.5 * (rhonp1[ijk2] + rhonp1[ijk2 + off]);
        u_int[ijk] = (rho1 * u[ijk] - const1 * h + const2 * hn[ijk]) / rhonp1_1;
        hn[ijk] = h;
    }
}

// conv_exitbc_scale (code/conv_exitbc_scale.F) of one variable's exit planes
// by (mflux_in - mass_change) / mflux_out
__global__ void k_exit_scale(const SideJob *__restrict__ jobs, int iva, double *__restrict__ f,
                             const double *__restrict__ ex)
{
    const SideJob J = jobs[blockIdx.x];
    if (!J.conv) return;
    const double scalef = (ex[EX_IN] - ex[EX_MCHG]) / ex[EX_OUT];
    const int *r = J.bnd[iva];
    const long n0 = J.n[0], ld = (long)J.n[0] * J.n[1];
    const bool low = (J.side % 2) == 1;
    long sa, sb, sc;
    int b0, b1, c0, c1, pa;
    // (d2, d3) = cyclic1 of d1: the loops run over the other two axes in
    // that order; the planes are the same whatever the loop order
    if (J.d1 == 1) {
        sa = 1; sb = n0; sc = ld; b0 = r[2]; b1 = r[3]; c0 = r[4]; c1 = r[5];
        pa = low ? r[0] - 1 : r[1] + 1;
    } else if (J.d1 == 2) {
        sa = n0; sb = 1; sc = ld; b0 = r[0]; b1 = r[1]; c0 = r[4]; c1 = r[5];
        pa = low ? r[2] - 1 : r[3] + 1;
    } else {
        sa = ld; sb = 1; sc = n0; b0 = r[0]; b1 = r[1]; c0 = r[2]; c1 = r[3];
        pa = low ? r[4] - 1 : r[5] + 1;
    }
    const int nb = b1 - b0 + 1, nc = c1 - c0 + 1;
    for (int q = threadIdx.x; q < nb * nc; q += blockDim.x) {
        const int bb = b0 + q % nb, cc = c0 + q / nb;
        const long ijk = J.off3 + sa * (pa - 1) + sb * (bb - 1) + sc * (cc - 1);
        f[ijk] = f[ijk] * scalef;
    }
}

// mass_change_block: per-CTA partial sums of (rhonp1 - rho) vol / dt over
// the interior, vol = rdidjp(i,j) dkw(k) (code/mass_change_block.F:53-64)
__global__ void __launch_bounds__(256) k_mass_change(const BlkDev *__restrict__ blk, double dtime,
                                                     const double *__restrict__ rho,
                                                     const double *__restrict__ rhonp1,
                                                     const double *__restrict__ rdidjp,
                                                     const double *__restrict__ dkw, double *__restrict__ partial)
{
    const BlkDev b = blk[blockIdx.y];
    const double ddtime = 1.0 / dtime;
    double v[1] = {0.};
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < b.ncell; t += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        const long p = decode_interior(b, t, i, j, k);
        const double vol = rdidjp[b.off2 + (i - 1) + (long)b.n[0] * (j - 1)] * dkw[b.off1k + k - 1];
        v[0] += ddtime * vol * (rhonp1[p] - rho[p]);
    }
    block_reduce_store<1>(v, partial + blockIdx.y * (long)gridDim.x + blockIdx.x);
}

// blocks' partials summed per block, then over blocks in block order
__global__ void k_mass_change_final(const double *__restrict__ partial, int gx, int nb, double *__restrict__ out)
{
    __shared__ double r[1];
    double total = 0.;
    for (int b = 0; b < nb; b++) {
        double v[1] = {0.};
        for (int t = threadIdx.x; t < gx; t += blockDim.x) v[0] += partial[(long)b * gx + t];
        block_reduce_store<1>(v, r);
        __syncthreads();
        total = total + r[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = total;
}

// counter-based uniform [0, 1): the splitmix64 finaliser of a key built
// from (seed, step, block, j, k), 53 bits
__device__ __forceinline__ double inlet_uniform(unsigned long long seed, int step, int block, int j, int k)
{
    unsigned long long key = seed;
    key = key * 0x9E3779B97F4A7C15ULL + (unsigned long long)(unsigned)step;
    key = key * 0x9E3779B97F4A7C15ULL + (unsigned long long)(unsigned)block;
    key = key * 0x9E3779B97F4A7C15ULL + (unsigned long long)(unsigned)j;
    key = key * 0x9E3779B97F4A7C15ULL + (unsigned long long)(unsigned)k;
    unsigned long long z = key;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// fixed_inlet (code/fixed_inlet.F:61-176) on one inlet block: the i = 2
// face and the i = 1 ghost cells, all j, k including ghosts
// step_dev (nullable): the step number read from device memory instead of
// step (a replayed graph: the host writes it before each launch)
__global__ void k_fixed_inlet(const BlkDev *__restrict__ blk, int iblk, int which, const double *__restrict__ uprof,
                              const double *__restrict__ vprof, unsigned long long seed, int step,
                              const int *__restrict__ step_dev, double rholo, double rhohi,
                              double *__restrict__ u, double *__restrict__ v,
                              double *__restrict__ w, double *__restrict__ sc1, double *__restrict__ rho,
                              double *__restrict__ u_int, double *__restrict__ v_int,
                              double *__restrict__ w_int)
{
    if (step_dev) step = *step_dev;
    const BlkDev b = blk[iblk];
    const int njp1 = b.n[1], nkp1 = b.n[2], nj = njp1 - 1;
    const long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    const int sh = (which - 1) * (nj - 1);
    const double amp = which <= 2 ? uprof[3 - 1] : uprof[4 * (nj - 2) - 1];
    const double fin = which <= 2 ? 0.0 : 1.0;
    const double rhoin = which <= 2 ? rholo : rhohi;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < njp1 * nkp1; q += gridDim.x * blockDim.x) {
        const int j = q % njp1 + 1, k = q / njp1 + 1;
        const double random = inlet_uniform(seed, step, iblk + 1, j, k);
        const double perturb = 0.005 * amp * 2.0 * (random - 0.5);
        const double uin = uprof[j + sh - 1] + perturb;
        const double vin = vprof[j + sh - 1] + perturb;
        const double win = perturb;
        const long ijk = b.off3 + 1 + jo * (j - 1) + ko * (k - 1), ijkw = ijk - 1;
        u[ijk] = uin;
        v[ijkw] = vin;
        w[ijkw] = win;
        sc1[ijkw] = fin;
        rho[ijkw] = rhoin;
        u_int[ijk] = uin;
        v_int[ijkw] = vin;
        w_int[ijkw] = win;
    }
}

// ---- recycling (mas-recyc/recycling.F) ----------------------------------
// plane averages over i = 2..nip1 of one block for every (j, k), j, k =
// 2..njp1 / nkp1 (pass 0: u, v, w; pass 1: their squared deviations from
// the running means), summed in the reference's order, one thread each
__global__ void k_recyc_work(const BlkDev *__restrict__ blk, int ib, int pass, const double *__restrict__ u,
                             const double *__restrict__ v, const double *__restrict__ w, const double *__restrict__ mu,
                             const double *__restrict__ mv, const double *__restrict__ mw, double *__restrict__ work)
{
    const BlkDev b = blk[ib];
    const int nip1 = b.n[0], njp1 = b.n[1], nkp1 = b.n[2];
    const long jo = nip1, ko = (long)nip1 * njp1;
    const int nj = njp1 - 1, nk = nkp1 - 1;
    const long plane = (long)(njp1 + 1) * (nkp1 + 1);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nj * nk; q += gridDim.x * blockDim.x) {
        const int j = 2 + q % nj, k = 2 + q / nj;
        const long base = b.off3 + jo * (j - 1) + ko * (k - 1);
        const double *f[3] = {u, v, w};
        const double *m[3] = {mu, mv, mw};
        for (int c = 0; c < 3; c++) {
            double s = 0.0;
            for (int i = 2; i <= nip1; i++) {
                double d = f[c][base + i - 1];
                if (pass == 1) {
                    d = d - m[c][j - 1];
                    d = d * d;
                }
                s = s + d;
            }
            work[c * plane + (long)k * (njp1 + 1) + j] = s / (double)(nip1 - 1);
        }
    }
}

// the running means (pass 0) or rms (pass 1) per j from the plane averages
__global__ void k_recyc_means(const BlkDev *__restrict__ blk, int ib, int pass, const double *__restrict__ work,
                              double *__restrict__ mu, double *__restrict__ mv, double *__restrict__ mw,
                              double *__restrict__ ru, double *__restrict__ rv, double *__restrict__ rw)
{
    const BlkDev b = blk[ib];
    const int njp1 = b.n[1], nkp1 = b.n[2];
    const long plane = (long)(njp1 + 1) * (nkp1 + 1);
    const double cpfilt = 0.144;
    double *m[3] = {mu, mv, mw}, *r[3] = {ru, rv, rw};
    for (int j = 2 + blockIdx.x * blockDim.x + threadIdx.x; j <= njp1; j += gridDim.x * blockDim.x)
        for (int c = 0; c < 3; c++) {
            double s = 0.0;
            for (int k = 2; k <= nkp1; k++) s = s + work[c * plane + (long)k * (njp1 + 1) + j];
            s = s / (double)(nkp1 - 1);
            if (pass == 0)
                m[c][j - 1] = cpfilt * s + (1. - cpfilt) * m[c][j - 1];
            else
                r[c][j - 1] = sqrt(cpfilt * s + (1. - cpfilt) * (r[c][j - 1] * r[c][j - 1]));
        }
}

// rescaling to the target mean and rms profiles (recycling.F:180-206)
__global__ void k_recyc_rescale(const BlkDev *__restrict__ blk, int ib, int i0, int jmult, RecycProf P,
                                double *__restrict__ u, double *__restrict__ v, double *__restrict__ w)
{
    const BlkDev b = blk[ib];
    const int nip1 = b.n[0], njp1 = b.n[1], nkp1 = b.n[2];
    const long jo = nip1, ko = (long)nip1 * njp1;
    const int ni = nip1 - i0 + 1, nj = njp1 - 1, nk = nkp1 - 1;
    const double small = 0.0000001;
    double *f[3] = {u, v, w};
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < (long)ni * nj * nk; q += (long)gridDim.x * blockDim.x) {
        const int i = i0 + (int)(q % ni), j = 2 + (int)((q / ni) % nj), k = 2 + (int)(q / ((long)ni * nj));
        const long ijk = b.off3 + (i - 1) + jo * (j - 1) + ko * (k - 1);
        for (int c = 0; c < 3; c++)
            f[c][ijk] = (P.rprof[c][j + jmult - 1] / (P.rms[c][j - 1] + small)) * (f[c][ijk] - P.mean[c][j - 1]) +
                        P.prof[c][j + jmult - 1];
    }
}

// the recycling plane (i = 3 for u, i = 2 for v, w) of block src, in (k, j)
// order, into the inflow plane of block dst (recycling.F:212-300)
__global__ void k_recyc_copy(const BlkDev *__restrict__ blk, int src, int dst, double rhohi, double *__restrict__ u,
                             double *__restrict__ v, double *__restrict__ w, double *__restrict__ sc1,
                             double *__restrict__ rho, double *__restrict__ u_int, double *__restrict__ v_int,
                             double *__restrict__ w_int)
{
    const BlkDev bs = blk[src], bd = blk[dst];
    const long ns = (long)(bs.n[1] - 1) * (bs.n[2] - 1), nd = (long)(bd.n[1] - 1) * (bd.n[2] - 1);
    const long n = ns < nd ? ns : nd;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int js = 2 + (int)(q % (bs.n[1] - 1)), ks = 2 + (int)(q / (bs.n[1] - 1));
        const int jd = 2 + (int)(q % (bd.n[1] - 1)), kd = 2 + (int)(q / (bd.n[1] - 1));
        const long is = bs.off3 + 2 + (long)bs.n[0] * (js - 1) + (long)bs.n[0] * bs.n[1] * (ks - 1);
        const long id = bd.off3 + 1 + (long)bd.n[0] * (jd - 1) + (long)bd.n[0] * bd.n[1] * (kd - 1);
        const double us = u[is], vs = v[is - 1], ws = w[is - 1];
        u[id] = us;
        v[id - 1] = vs;
        w[id - 1] = ws;
        sc1[id - 1] = 1.0;
        rho[id - 1] = rhohi;
        u_int[id] = us;
        v_int[id - 1] = vs;
        w_int[id - 1] = ws;
    }
}

// ---- span-averaged statistics (code/statistics.F) ------------------------
// cell-centred velocities of one block as statistics.F's centre makes them:
// the interior, then the i, k and j boundary planes; edge cells stay 0
__global__ void k_centre(const BlkDev *__restrict__ blk, const double *__restrict__ u, const double *__restrict__ v,
                         const double *__restrict__ w, double *__restrict__ ut, double *__restrict__ vt,
                         double *__restrict__ wt)
{
    const BlkDev b = blk[blockIdx.y];
    const int nip1 = b.n[0], njp1 = b.n[1], nkp1 = b.n[2];
    const long jo = nip1, ko = (long)nip1 * njp1, np = (long)nip1 * njp1 * nkp1;
    const double *U = u + b.off3, *V = v + b.off3, *W = w + b.off3;
    double *Ut = ut + b.off3, *Vt = vt + b.off3, *Wt = wt + b.off3;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < np; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nip1) + 1, j = (int)((q / nip1) % njp1) + 1, k = (int)(q / ko) + 1;
        const long p = q;  // 0-based ijk - 1
        const bool ii = i >= 2 && i <= nip1 - 1, jj = j >= 2 && j <= njp1 - 1, kk = k >= 2 && k <= nkp1 - 1;
        double a = 0., bv = 0., cw = 0.;
        if (ii && jj && kk) {
            a = 0.5 * (U[p] + U[p + 1]);
            bv = 0.5 * (V[p] + V[p + jo]);
            cw = 0.5 * (W[p] + W[p + ko]);
        } else if (jj && kk && i == 1) {
            a = U[p + 1];
            bv = 0.25 * (V[p] + V[p + 1] + V[p + jo] + V[p + jo + 1]);
            cw = 0.25 * (W[p] + W[p + 1] + W[p + ko] + W[p + ko + 1]);
        } else if (jj && kk && i == nip1) {
            a = U[p];
            bv = 0.25 * (V[p] + V[p - 1] + V[p + jo] + V[p + jo - 1]);
            cw = 0.25 * (W[p] + W[p - 1] + W[p + ko] + W[p + ko - 1]);
        } else if (ii && jj && k == 1) {
            cw = W[p + ko];
            bv = 0.25 * (V[p] + V[p + ko] + V[p + jo] + V[p + jo + ko]);
            a = 0.25 * (U[p] + U[p + ko] + U[p + 1] + U[p + ko + 1]);
        } else if (ii && jj && k == nkp1) {
            cw = W[p];
            bv = 0.25 * (V[p] + V[p - ko] + V[p + jo] + V[p + jo - ko]);
            a = 0.25 * (U[p] + U[p - ko] + U[p + 1] + U[p - ko + 1]);
        } else if (ii && kk && j == 1) {
            bv = V[p + jo];
            cw = 0.25 * (W[p] + W[p + jo] + W[p + ko] + W[p + ko + jo]);
            a = 0.25 * (U[p] + U[p + jo] + U[p + 1] + U[p + jo + 1]);
        } else if (ii && kk && j == njp1) {
            bv = V[p];
            cw = 0.25 * (W[p] + W[p - jo] + W[p + ko] + W[p + ko - jo]);
            a = 0.25 * (U[p] + U[p - jo] + U[p + 1] + U[p - jo + 1]);
        }
        Ut[p] = a;
        Vt[p] = bv;
        Wt[p] = cw;
    }
}

// the 16 span means (k = 2..nkp1-1, in order) of one (i, j) column folded
// into the running averages over no_sam samples
__global__ void k_span_stats(const BlkDev *__restrict__ blk, int no_sam, const double *__restrict__ ut,
                             const double *__restrict__ vt, const double *__restrict__ wt,
                             const double *__restrict__ p, const double *__restrict__ rho,
                             const double *__restrict__ sc1, const double *__restrict__ sc1var,
                             const double *__restrict__ gam, StatOut O)
{
    const BlkDev b = blk[blockIdx.y];
    const int nip1 = b.n[0], njp1 = b.n[1], nkp1 = b.n[2];
    const long jo = nip1, ko = (long)nip1 * njp1;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < (long)nip1 * njp1;
         q += (long)gridDim.x * blockDim.x) {
        double s[16];
        for (int m = 0; m < 16; m++) s[m] = 0.0;
        for (int k = 2; k <= nkp1 - 1; k++) {
            const long ijk = b.off3 + q + ko * (k - 1);
            const double rr = rho[ijk], uu = ut[ijk], vv = vt[ijk], ww = wt[ijk];
            s[0] = s[0] + rr * uu;
            s[1] = s[1] + rr * vv;
            s[2] = s[2] + rr * ww;
            s[3] = s[3] + p[ijk];
            s[4] = s[4] + rr;
            s[5] = s[5] + rr * uu * vv;
            s[6] = s[6] + rr * vv * ww;
            s[7] = s[7] + rr * uu * ww;
            s[8] = s[8] + rr * uu * uu;
            s[9] = s[9] + rr * vv * vv;
            s[10] = s[10] + rr * ww * ww;
            s[11] = s[11] + rr * rr;
            s[12] = s[12] + sc1[ijk];
            s[13] = s[13] + sc1[ijk] * sc1[ijk];
            s[14] = s[14] + sc1var[ijk];
            s[15] = s[15] + gam[ijk];
        }
        (void)jo;
        const long ij = b.off2 + q;
        for (int m = 0; m < 16; m++) {
            const double avg = s[m] / (double)(nkp1 - 2);
            O.f[m][ij] = (O.f[m][ij] * (double)(no_sam - 1) + avg) / (double)no_sam;
        }
    }
}

// ================================================================ launchers
namespace les {

void launch_side_flux(const SideJob *jobs, int njobs, int iva, int which, const double *u, const double *v,
                      const double *w, const double *rho, const double *rdju, const double *rdiv,
                      const double *didjp, const double *dkp, double *out, cudaStream_t st)
{
    if (njobs == 0) return;
    k_side_flux<<<njobs, 256, 0, st>>>(jobs, iva, which, u, v, w, rho, rdju, rdiv, didjp, dkp, out);
    count_launch(1);
}

void launch_side_combine(const SideJob *jobs, int njobs, const double *out, int mode, double *ex,
                         cudaStream_t st)
{
    k_side_combine<<<1, 32, 0, st>>>(jobs, njobs, out, mode, ex);
    count_launch(1);
}

void launch_exit_update(const SideJob *jobs, int njobs, int task, int iva, const ExitMetrics &M, double *u,
                        double *u_int, const double *rho, const double *rhonp1, double *hn, double dtime,
                        const double *ex, cudaStream_t st)
{
    if (njobs == 0) return;
    k_exit_update<<<njobs, 256, 0, st>>>(jobs, task, iva, M, u, u_int, rho, rhonp1, hn, dtime, ex);
    count_launch(1);
}

void launch_exit_scale(const SideJob *jobs, int njobs, int iva, double *f, const double *ex, cudaStream_t st)
{
    if (njobs == 0) return;
    k_exit_scale<<<njobs, 256, 0, st>>>(jobs, iva, f, ex);
    count_launch(1);
}

void launch_mass_change(const BlkDev *blk, int nb, long maxcell, double dtime, const double *rho,
                        const double *rhonp1, const double *rdidjp, const double *dkw, double *partial,
                        double *out, cudaStream_t st)
{
    unsigned gx = (unsigned)((maxcell + 255) / 256);
    unsigned cap = (unsigned)((1216 + nb - 1) / nb);
    if (gx > cap) gx = cap;
    k_mass_change<<<dim3(gx, nb), 256, 0, st>>>(blk, dtime, rho, rhonp1, rdidjp, dkw, partial);
    k_mass_change_final<<<1, 256, 0, st>>>(partial, (int)gx, nb, out);
    count_launch(2);
}

void launch_fixed_inlet(const BlkDev *blk, int iblk, int which, int nplane, const double *uprof,
                        const double *vprof, unsigned long long seed, int step, const int *step_dev, double rholo,
                        double rhohi, double *u, double *v, double *w, double *sc1, double *rho, double *u_int,
                        double *v_int, double *w_int, cudaStream_t st)
{
    unsigned g = (unsigned)((nplane + 255) / 256);
    k_fixed_inlet<<<g, 256, 0, st>>>(blk, iblk, which, uprof, vprof, seed, step, step_dev, rholo, rhohi, u, v, w,
                                     sc1, rho, u_int, v_int, w_int);
    count_launch(1);
}

void launch_statistics(const BlkDev *blk, int nb, long maxpts, long maxij, int no_sam, const double *u,
                       const double *v, const double *w, const double *p, const double *rho, const double *sc1,
                       const double *sc1var, const double *gam, double *ut, double *vt, double *wt,
                       const StatOut &O, cudaStream_t st)
{
    unsigned g1 = (unsigned)((maxpts + 255) / 256), g2 = (unsigned)((maxij + 127) / 128);
    k_centre<<<dim3(g1 > 2048 ? 2048 : g1, nb), 256, 0, st>>>(blk, u, v, w, ut, vt, wt);
    k_span_stats<<<dim3(g2, nb), 128, 0, st>>>(blk, no_sam, ut, vt, wt, p, rho, sc1, sc1var, gam, O);
    count_launch(2);
}

void launch_recycling(const BlkDev *blk, const int *nijk, int nb, int step, int inblock, int jmult, double rhohi,
                      const RecycProf &P, double *u, double *v, double *w, double *sc1, double *rho, double *u_int,
                      double *v_int, double *w_int, double *work, cudaStream_t st)
{
    for (int b = inblock; b <= inblock + 7 && b <= nb; b++) {
        const int *n = nijk + 3 * (b - 1);
        unsigned g = (unsigned)(((long)(n[1] - 1) * (n[2] - 1) + 255) / 256);
        for (int pass = 0; pass < 2; pass++) {
            k_recyc_work<<<g, 256, 0, st>>>(blk, b - 1, pass, u, v, w, P.mean[0], P.mean[1], P.mean[2], work);
            k_recyc_means<<<(unsigned)((n[1] + 127) / 128), 128, 0, st>>>(
                blk, b - 1, pass, work, (double *)P.mean[0], (double *)P.mean[1], (double *)P.mean[2],
                (double *)P.rms[0], (double *)P.rms[1], (double *)P.rms[2]);
            count_launch(2);
        }
    }
    for (int b = inblock; b <= inblock + 7 && b <= nb; b++) {
        if (!(step % 100 == 0 && step >= 200)) break;
        const int *n = nijk + 3 * (b - 1);
        int i0 = b != inblock ? 1 : 2;
        long cnt = (long)(n[0] - i0 + 1) * (n[1] - 1) * (n[2] - 1);
        unsigned g = (unsigned)((cnt + 255) / 256);
        k_recyc_rescale<<<g > 4096 ? 4096 : g, 256, 0, st>>>(blk, b - 1, i0, jmult, P, u, v, w);
        count_launch(1);
    }
    if (inblock + 7 <= nb) {
        const int *n = nijk + 3 * (inblock - 1);
        unsigned g = (unsigned)(((long)(n[1] - 1) * (n[2] - 1) + 255) / 256);
        k_recyc_copy<<<g, 256, 0, st>>>(blk, inblock + 6, inblock - 1, rhohi, u, v, w, sc1, rho, u_int, v_int, w_int);
        count_launch(1);
    }
}

} // namespace les
