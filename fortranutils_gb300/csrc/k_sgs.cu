// k_sgs.cu -- eddy-viscosity kernels (FP64; exact and fast builds, see
// phys_variant.h), one thread per interior point of every block.
//
// subgrid (code/subgrid.F:58-92) dispatches on the model:
//   Smagorinsky  code/subgrid_smagorinsky.F:85-237
//   WALE         code/subgrid_wale.F:73-239 (the reference's scalar Sd)
//   Sigma        edge/subgrid_sigma.F:66-300 (model 3 of the reference's edge
//                variant): singular values of the gradient tensor from the
//                invariants of g = grad(u)^T grad(u) by the trigonometric
//                cubic solution.  As written there, the square root in the
//                eigenvalue formula is taken of the COMMON `alpha` (the density
//                relaxation factor of cb.control.inc), not of alpha1; that is
//                reproduced: with alpha = 0 the three values coincide and gam
//                is 0.
//   none         code/subgrid_nosgs.F (gam = gamsc1 = 0)
// The staggered-grid gradients are the reference's face/edge averages.  The
// filter width uses the reference's literal exponent 0.33333333.  pow() is
// CUDA's and may differ from a CPU libm in the last bit; everything else is
// operation-for-operation.
#include "k_common.cuh"
#include "kernels.h"
#include "phys_variant.h"

namespace LES_PHYS_NS {

#define IDX2(b, i, j) ((b).off2 + ((i) - 1) + (long)(b).n[0] * ((j) - 1))

__global__ void __launch_bounds__(128) k_subgrid(
    const BlkDev *__restrict__ blk, int model, double csles, int gotrad, double alpha,
    double *__restrict__ gam, double *__restrict__ gamsc1, const double *__restrict__ u,
    const double *__restrict__ v, const double *__restrict__ w, const double *__restrict__ sc1,
    double *__restrict__ sc1var, double *__restrict__ sc1dis, const double *__restrict__ vdd,
    const double *__restrict__ dip, const double *__restrict__ diu, const double *__restrict__ djp,
    const double *__restrict__ djv, const double *__restrict__ dkp, const double *__restrict__ dkw,
    const double *__restrict__ hijp, const double *__restrict__ hjip,
    const double *__restrict__ hkip, const double *__restrict__ hkjp, const double *__restrict__ rp,
    SgsFast F)
{
    (void)F;
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long ijk = decode_interior(b, q, i, j, k);
    if (model == 0) {
        gam[ijk] = 0.0;
        gamsc1[ijk] = 0.0;
        sc1var[ijk] = 0.0;
        sc1dis[ijk] = 0.0;
        return;
    }
    const double sct = 0.3, cfv = 0.1;
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    long ijkw = ijk - 1, ijke = ijk + 1, ijks = ijk - jo, ijkn = ijk + jo, ijkl = ijk - ko,
         ijkr = ijk + ko;
    long ijkse = ijks + 1, ijknw = ijkn - 1, ijkne = ijkn + 1, ijkel = ijke - ko, ijknl = ijkn - ko,
         ijkwr = ijkw + ko, ijker = ijke + ko, ijksr = ijks + ko, ijknr = ijkn + ko;
    long ij = IDX2(b, i, j);
    double dkwk = dkw[b.off1k + k - 1], dkpk = dkp[b.off1k + k - 1];
#ifdef LES_FAST_PHYS
    const double rdi = F.r_dip[ij], rdj = F.r_djp[ij], rdkp = F.r_dkp[b.off1k + k - 1];
#endif

    double fwf = 0.5 * (sc1[ijk] + sc1[ijkw]);
    double fef = 0.5 * (sc1[ijk] + sc1[ijke]);
    double fsf = 0.5 * (sc1[ijk] + sc1[ijks]);
    double fnf = 0.5 * (sc1[ijk] + sc1[ijkn]);
    double flf = 0.5 * (sc1[ijk] + sc1[ijkl]);
    double frf = 0.5 * (sc1[ijk] + sc1[ijkr]);
    double dfdip = QDIV(fef - fwf, dip[ij], rdi);
    double dfdjp = QDIV(fnf - fsf, djp[ij], rdj);
    double dfdkp = QDIV(frf - flf, (rp[ij] * dkwk), F.r_rp[ij] * F.r_dkw[b.off1k + k - 1]);

    double up = 0.5 * (u[ijk] + u[ijke]);
    double vp = 0.5 * (v[ijk] + v[ijkn]);
    double di = dip[ij], dj = djp[ij], dk;
    double vwf = 0.25 * (v[ijk] + v[ijkn] + v[ijkw] + v[ijknw]);
    double vef = 0.25 * (v[ijk] + v[ijkn] + v[ijke] + v[ijkne]);
    double usf = 0.25 * (u[ijk] + u[ijke] + u[ijks] + u[ijkse]);
    double unf = 0.25 * (u[ijk] + u[ijke] + u[ijkn] + u[ijkne]);
    double ulf = 0.25 * (u[ijk] + u[ijke] + u[ijkl] + u[ijkel]);
    double urf = 0.25 * (u[ijk] + u[ijke] + u[ijkr] + u[ijker]);
    double vlf = 0.25 * (v[ijk] + v[ijkn] + v[ijkl] + v[ijknl]);
    double vrf = 0.25 * (v[ijk] + v[ijkn] + v[ijkr] + v[ijknr]);

    double dudi = QDIV(u[ijke] - u[ijk], di, rdi) + vp * hijp[ij];
    double dvdi = QDIV(vef - vwf, di, rdi) - up * hijp[ij];
    double dudj = QDIV(unf - usf, dj, rdj) - vp * hjip[ij];
    double dvdj = QDIV(v[ijkn] - v[ijk], dj, rdj) + up * hjip[ij];
    double dwdi, dwdj, dudk, dvdk, dwdk;
    if (gotrad) {
        long jn = b.n[0];
        double radp = rp[ij], radw = rp[ij - 1], rade = rp[ij + 1], rads = rp[ij - jn],
               radn = rp[ij + jn];
        dk = radp * dkpk;
        double hki = hkip[ij], hkj = hkjp[ij];
        double wdrw = 0.5 * (w[ijkw] + w[ijkwr]) / radw;
        double wdre = 0.5 * (w[ijke] + w[ijker]) / rade;
        double wdrs = 0.5 * (w[ijks] + w[ijksr]) / rads;
        double wdrn = 0.5 * (w[ijkn] + w[ijknr]) / radn;
        dwdi = radp * (wdre - wdrw) / (diu[ij] + diu[ij + 1]);
        dwdj = radp * (wdrn - wdrs) / (djv[ij] + djv[ij + jn]);
        double wp = 0.5 * (w[ijk] + w[ijkr]);
#ifdef LES_FAST_PHYS
        const double rdk = F.r_rp[ij] * rdkp;
#endif
        dudk = QDIV(urf - ulf, dk, rdk) - wp * hki;
        dvdk = QDIV(vrf - vlf, dk, rdk) - wp * hkj;
        dwdk = QDIV(w[ijkr] - w[ijk], dk, rdk) + up * hki + vp * hkj;
    } else {
        dk = dkpk;
        double wwf = 0.25 * (w[ijk] + w[ijkr] + w[ijkw] + w[ijkwr]);
        double wef = 0.25 * (w[ijk] + w[ijkr] + w[ijke] + w[ijker]);
        double wsf = 0.25 * (w[ijk] + w[ijkr] + w[ijks] + w[ijksr]);
        double wnf = 0.25 * (w[ijk] + w[ijkr] + w[ijkn] + w[ijknr]);
        dwdi = QDIV(wef - wwf, di, rdi);
        dwdj = QDIV(wnf - wsf, dj, rdj);
        dudk = QDIV(urf - ulf, dk, rdkp);
        dvdk = QDIV(vrf - vlf, dk, rdkp);
        dwdk = QDIV(w[ijkr] - w[ijk], dk, rdkp);
    }
    double sijsij = dvdj * dvdj + dwdk * dwdk + dudi * dudi +
                    0.5 * ((dudj + dvdi) * (dudj + dvdi) + (dvdk + dwdj) * (dvdk + dwdj) +
                           (dudk + dwdi) * (dudk + dwdi));
#ifdef LES_FAST_PHYS
    // (di dj dk)^e = (dip djp rp)^e dkp^e: rp is 1 exactly off polar grids
    double delta_xyz = F.delta2d[ij] * F.delta1d[b.off1k + k - 1];
#else
    double delta_xyz = pow(di * dj * dk, .33333333);
#endif
    double g;
    if (model == 1) {
        double evisc = csles * delta_xyz * vdd[ijk];
        g = evisc * evisc * sqrt(2.0 * sijsij);
    } else if (model == 3) {
        const double onethird = 1.0 / 3.0, pi = 3.1415927;
        double g11 = dudi * dudi + dvdi * dvdi + dwdi * dwdi;
        double g12 = dudi * dudj + dvdi * dvdj + dwdi * dwdj;
        double g13 = dudi * dudk + dvdi * dvdk + dwdi * dwdk;
        double g21 = dudj * dudi + dvdj * dvdi + dwdj * dwdi;
        double g22 = dudj * dudj + dvdj * dvdj + dwdj * dwdj;
        double g23 = dudj * dudk + dvdj * dvdk + dwdj * dwdk;
        double g31 = dudk * dudi + dvdk * dvdi + dwdk * dwdi;
        double g32 = dudk * dudj + dvdk * dvdj + dwdk * dwdj;
        double g33 = dudk * dudk + dvdk * dvdk + dwdk * dwdk;
        double gg11 = g11 * g11 + g12 * g21 + g13 * g31;
        double gg22 = g21 * g12 + g22 * g22 + g23 * g32;
        double gg33 = g31 * g13 + g32 * g23 + g33 * g33;
        double tracegg = gg11 + gg22 + gg33;
        double inv1 = g11 + g22 + g33;
        double inv2 = 0.5 * (inv1 * inv1 - tracegg);
        double inv3 = g11 * (g22 * g33 - g23 * g32) - g12 * (g21 * g33 - g23 * g31) + g13 * (g21 * g32 - g22 * g31);
        double alpha1 = (inv1 * inv1 * 0.11111111) - (inv2 * onethird);
        double alpha2 = (inv1 * inv1 * inv1 * 0.03703703703) - (inv1 * inv2 * 0.16666666666) + (inv3 * 0.5);
        double alpha3 = onethird * acos(alpha2 / pow(alpha1, 1.5));
        double inv13 = inv1 * onethird;
        double sqrtalpha = sqrt(alpha);
        double sigma1 = pow(inv13 + 2.0 * sqrtalpha * cos(alpha3), 0.5);
        double sigma2 = pow(inv13 - 2.0 * sqrtalpha * cos(pi * onethird + alpha3), 0.5);
        double sigma3 = pow(inv13 - 2.0 * sqrtalpha * cos(pi * onethird - alpha3), 0.5);
        double sigmafinal = (sigma3 * (sigma1 - sigma2) * (sigma2 - sigma3)) / pow(sigma1, 2.0);
        double evisc = (csles * delta_xyz) * (csles * delta_xyz);
        g = evisc * sigmafinal;
    } else {
        double g11 = dudi * dudi + dudj * dvdi + dudk * dwdi;
        double g22 = dvdi * dudj + dvdj * dvdj + dvdk * dwdj;
        double g33 = dwdi * dudk + dwdj * dvdk + dwdk * dwdk;
        double g12 = dudi * dudj + dudj * dvdj + dudk * dwdj;
        double g13 = dudi * dudk + dudj * dvdk + dudk * dwdk;
        double g21 = dvdi * dudi + dvdj * dvdi + dvdk * dwdi;
        double g23 = dvdi * dudk + dvdj * dvdk + dvdk * dwdk;
        double g31 = dwdi * dudi + dwdj * dvdi + dwdk * dwdi;
        double g32 = dwdi * dudj + dwdj * dvdj + dwdk * dwdj;
        double tracet = (1.0 / 3.0) * (g11 + g22 + g33);
        double sdij = (g11 - tracet) + (g22 - tracet) + (g33 - tracet) + 0.5 * (g12 + g21) +
                      0.5 * (g13 + g31) + 0.5 * (g23 + g32);
        double sd2 = sdij * sdij;
        double ev = (csles * delta_xyz) * (csles * delta_xyz);
#ifdef LES_FAST_PHYS
        // x^1.5 = x sqrt(x), x^2.5 = x^2 sqrt(x), x^1.25 = x sqrt(sqrt(x)) for x >= 0
        double rsd = sqrt(sd2), rss = sqrt(sijsij);
        g = ev * ((sd2 * rsd) / (sijsij * sijsij * rss + sd2 * sqrt(rsd)));
#else
        g = ev * (pow(sd2, 1.5) / (pow(sijsij, 2.5) + pow(sd2, 1.25)));
#endif
    }
    gam[ijk] = g;
    gamsc1[ijk] = (csles == 0.0) ? 0.0 : g / sct;
    double dfdijk = dfdip * dfdip + dfdjp * dfdjp + dfdkp * dfdkp;
    double sv = cfv * dfdijk * (delta_xyz * delta_xyz);
    sc1var[ijk] = sv;
    sc1dis[ijk] = sv * sqrt(2.0 * sijsij);
}

void launch_subgrid(const BlkDev *blk, int nb, long maxcell, int model, double csles, int gotrad,
                    double alpha, double *gam, double *gamsc1, const double *u, const double *v, const double *w,
                    const double *sc1, double *sc1var, double *sc1dis, const double *vdd,
                    const double *const *m, const SgsFast &f, cudaStream_t st)
{
    // m: dip, diu, djp, djv, dkp, dkw, hijp, hjip, hkip, hkjp, rp
    k_subgrid<<<dim3((unsigned)((maxcell + 127) / 128), nb), 128, 0, st>>>(
        blk, model, csles, gotrad, alpha, gam, gamsc1, u, v, w, sc1, sc1var, sc1dis, vdd, m[0], m[1], m[2],
        m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], f);
    les::count_launch(1);
}

} // namespace LES_PHYS_NS
