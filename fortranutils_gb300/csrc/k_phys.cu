// k_phys.cu -- momentum predictor and scalar transport (FP64; exact and fast
// builds, see phys_variant.h).
//
//   set_u_int_block  code/set_u_int_block.F:103-462 (u, and v with the i/j
//                    roles swapped exactly as set_uv_int passes them)
//   set_w_int_block  code/set_w_int_block.F:95-458
//   set_gamsc1_bc    code/set_gamsc1_bc.F
//   set_sc1_block    code/set_sc1_block.F:66-505 -- sc1 is updated in place
//                    in the loop order j, i, k, so every point reads new
//                    values at its -1/-2 neighbours on each axis and old
//                    values at +1/+2.  Points of one hyperplane i+j+k = s
//                    are independent, so sweeping s upward reproduces the
//                    reference's result exactly.
//   set_sc1_bc       code/set_sc1_bc.F
//   set_sc1var_block code/set_sc1var_block.F:26-66
#include <cuda/atomic>

#include "k_common.cuh"
#include "kernels.h"
#include "phys_variant.h"

namespace LES_PHYS_NS {

#define IDX2(b, i, j) ((b).off2 + ((i) - 1) + (long)(b).n[0] * ((j) - 1))

// ------------------------------------------------------------- predictor
// u (iva = 1): nip1, njp1 = n[0], n[1]; io = 1, jo = n[0].
// v (iva = 2): nip1, njp1 = n[1], n[0]; io = n[0], jo = 1 (set_uv_int.F:119-142).
__global__ void __launch_bounds__(128) k_set_u_int(const BlkDev *__restrict__ blk, int iva,
                                                   UIntArgs A_, double dtime, int iststep,
                                                   double visc, double ylaminar, double kappa,
                                                   double cwfun)
{
    if (A_.iststep) iststep = *A_.iststep;
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int ir, jr, k;
    long ijk = decode_interior(b, q, ir, jr, k);
    int i = iva == 1 ? ir : jr, j = iva == 1 ? jr : ir;
    int nip1 = iva == 1 ? b.n[0] : b.n[1], njp1 = iva == 1 ? b.n[1] : b.n[0], nkp1 = b.n[2];
    long io = iva == 1 ? 1 : b.n[0], jo = iva == 1 ? b.n[0] : 1, ko = (long)b.n[0] * b.n[1];
    long io_ij = io, jo_ij = jo;
    // first side of the i axis and of the j axis (selects, not an index:
    // a runtime index would put the descriptor copy in local memory)
    int s0 = iva == 1 ? b.bc[0] : b.bc[2];
    int istart = (s0 != LES_BCT_PERIODIC_D && s0 != LES_BCT_INTERFACE_D) ? 3 : 2;
    if (i < istart) return;
    bool wallsf = (iva == 1 ? b.bc[2] : b.bc[0]) == LES_BCT_WALL_D;
    bool wallnf = (iva == 1 ? b.bc[3] : b.bc[1]) == LES_BCT_WALL_D;
    bool walllf = b.bc[4] == LES_BCT_WALL_D, wallrf = b.bc[5] == LES_BCT_WALL_D;
    int nj = njp1 - 1, nk = nkp1 - 1;
    double st1 = iststep - 1, st2 = iststep - 2, stden = 1.0 / iststep;
    const double *u = A_.u, *v = A_.v, *w = A_.w, *rho = A_.rho, *gam = A_.gam;
    long o2 = b.off2;
    // 0-based 2-D positions of ij, ijw, ijs, ijn, ijnw
    long ij = o2 + io_ij * (i - 1) + jo_ij * (j - 1);
    long ijw = ij - io_ij, ijs = ij - jo_ij, ijn = ij + jo_ij, ijnw = ijw + jo_ij;
    long ki = b.off1k * 0 + (k - 1) + (long)nkp1 * (i - 1);  // (k, i) of this block's wall array
    const double *dkp = A_.dkp + b.off1k, *dkw = A_.dkw + b.off1k;
#ifdef LES_FAST_PHYS
    const double *rdkp_ = A_.r_dkp + b.off1k, *rdkw_ = A_.r_dkw + b.off1k;
#endif
    double di = A_.diu[ij], dj = A_.dju[ij];
    long ijkw = ijk - io, ijke = ijk + io, ijks = ijk - jo, ijkn = ijk + jo, ijkl = ijk - ko, ijkr = ijk + ko;
    long ijksw = ijks - io, ijknw = ijkn - io, ijkwl = ijkw - ko, ijkwr = ijkw + ko;
    double rdkp = A_.rp[ij] * dkp[k - 1];
    double rdku = A_.ru[ij] * dkp[k - 1];
    double va = 0.25 * (v[ijk] + v[ijkn] + v[ijkw] + v[ijknw]);
    double wa = 0.25 * (w[ijk] + w[ijkr] + w[ijkw] + w[ijkwr]);
    double rhoa = 0.5 * (rho[ijkw] + rho[ijk]);
    double gama = 0.5 * (gam[ijkw] + gam[ijk]);
    double rhowf = rho[ijkw], rhoef = rho[ijk];
    double rhosf = 0.25 * (rho[ijk] + rho[ijkw] + rho[ijks] + rho[ijksw]);
    double rhonf = 0.25 * (rho[ijk] + rho[ijkw] + rho[ijkn] + rho[ijknw]);
    double rholf = 0.25 * (rho[ijk] + rho[ijkw] + rho[ijkl] + rho[ijkwl]);
    double rhorf = 0.25 * (rho[ijk] + rho[ijkw] + rho[ijkr] + rho[ijkwr]);
    double rhou = 0.5 * (rho[ijk] + rho[ijkw]);
    double rhonp1u = 0.5 * (A_.rhonp1[ijk] + A_.rhonp1[ijkw]);
    double gamwf = visc + gam[ijkw] * rhowf;
    double gamef = visc + gam[ijk] * rhoef;
    double gamsf = visc + .25 * (gam[ijk] + gam[ijkw] + gam[ijks] + gam[ijksw]) * rhosf;
    double gamnf = visc + .25 * (gam[ijk] + gam[ijkw] + gam[ijkn] + gam[ijknw]) * rhonf;
    double gamlf = visc + .25 * (gam[ijk] + gam[ijkw] + gam[ijkl] + gam[ijkwl]) * rholf;
    double gamrf = visc + .25 * (gam[ijk] + gam[ijkw] + gam[ijkr] + gam[ijkwr]) * rhorf;
    double areawf = A_.rdjp[ijw] * dkp[k - 1];
    double areaef = A_.rdjp[ij] * dkp[k - 1];
    double areasf = A_.rdix[ij] * dkp[k - 1];
    double areanf = A_.rdix[ijn] * dkp[k - 1];
    double areak = A_.didju[ij];
    double vol = A_.rdidju[ij] * dkp[k - 1];
    double uwf = 0.5 * (u[ijk] + u[ijkw]);
    double uef = 0.5 * (u[ijk] + u[ijke]);
    double vsf = 0.5 * (v[ijk] + v[ijkw]);
    double vnf = 0.5 * (v[ijkn] + v[ijknw]);
    double wlf = 0.5 * (w[ijk] + w[ijkw]);
    double wrf = 0.5 * (w[ijkr] + w[ijkwr]);
    double gwf = uwf * uwf * rhowf * areawf;
    double gef = uef * uef * rhoef * areaef;
    double gsf = 0.5 * (u[ijk] + u[ijks]) * vsf * rhosf * areasf;
    double gnf = 0.5 * (u[ijk] + u[ijkn]) * vnf * rhonf * areanf;
    double glf = 0.5 * (u[ijk] + u[ijkl]) * wlf * rholf * areak;
    double grf = 0.5 * (u[ijk] + u[ijkr]) * wrf * rhorf * areak;
    double conf = -(gef - gwf) - (gnf - gsf) - (grf - glf);
    double cc1 = A_.hjiu[ij] * rhoa * (va * va) * vol;
    double cc2 = A_.hkiu[ij] * rhoa * (wa * wa) * vol;
    double cc3 = -A_.hiju[ij] * rhoa * va * u[ijk] * vol;
    double conc = cc1 + cc2 + cc3;
    double galwf = QDIV(gamwf * areawf, A_.dip[ijw], A_.r_dip[ijw]);
    double galef = QDIV(gamef * areaef, A_.dip[ij], A_.r_dip[ij]);
    double galsf = QDIV(gamsf * areasf, A_.djx[ij], A_.r_djx[ij]);
    double galnf = QDIV(gamnf * areanf, A_.djx[ijn], A_.r_djx[ijn]);
    double gallf = QDIV(gamlf * areak, (A_.rp[ij] * dkw[k - 1]), A_.r_rp[ij] * rdkw_[k - 1]);
    double galrf = QDIV(gamrf * areak, (A_.rp[ij] * dkw[k]), A_.r_rp[ij] * rdkw_[k]);
    double vwf = 0.5 * (v[ijkw] + v[ijknw]);
    double vef = 0.5 * (v[ijk] + v[ijkn]);
    double twf = galwf * 2.0 * (u[ijk] - u[ijkw]);
    double tef = galef * 2.0 * (u[ijke] - u[ijk]);
    double tsf = galsf * A_.dix[ij] *
                 (QDIV(u[ijk], A_.diu[ij], A_.r_diu[ij]) - QDIV(u[ijks], A_.diu[ijs], A_.r_diu[ijs]));
    double tnf = galnf * A_.dix[ijn] *
                 (QDIV(u[ijkn], A_.diu[ijn], A_.r_diu[ijn]) - QDIV(u[ijk], A_.diu[ij], A_.r_diu[ij]));
    double tlf = gallf * (u[ijk] - u[ijkl]);
    double trf = galrf * (u[ijkr] - u[ijk]);
    double cwf = 2.0 * gamwf * areawf * vwf * A_.hijp[ijw];
    double cef = 2.0 * gamef * areaef * vef * A_.hijp[ij];
    double csf = QDIV(gamsf * areasf * A_.djx[ij] *
                          (QDIV(v[ijk], A_.djv[ij], A_.r_djv[ij]) - QDIV(v[ijkw], A_.djv[ijw], A_.r_djv[ijw])),
                      A_.dix[ij], A_.r_dix[ij]);
    double cnf = QDIV(gamnf * areanf * A_.djx[ijn] *
                          (QDIV(v[ijkn], A_.djv[ijn], A_.r_djv[ijn]) -
                           QDIV(v[ijknw], A_.djv[ijnw], A_.r_djv[ijnw])),
                      A_.dix[ijn], A_.r_dix[ijn]);
    double clf = QDIV(gamlf * areak * A_.ru[ij] *
                          (QDIV(w[ijk], A_.rp[ij], A_.r_rp[ij]) - QDIV(w[ijkw], A_.rp[ijw], A_.r_rp[ijw])),
                      A_.diu[ij], A_.r_diu[ij]);
    double crf = QDIV(gamrf * areak * A_.ru[ij] *
                          (QDIV(w[ijkr], A_.rp[ij], A_.r_rp[ij]) - QDIV(w[ijkwr], A_.rp[ijw], A_.r_rp[ijw])),
                      A_.diu[ij], A_.r_diu[ij]);
    double tiiwf = twf + cwf, tiief = tef + cef, tjisf = tsf + csf, tjinf = tnf + cnf;
    double tkilf = tlf + clf, tkirf = trf + crf;
    vsf = 0.5 * (v[ijk] + v[ijkw]);
    vnf = 0.5 * (v[ijkn] + v[ijknw]);
    double dc1 = -2.0 * gama * vol * A_.hjiu[ij] * (QDIV(vnf - vsf, A_.dju[ij], A_.r_dju[ij]) + u[ijk] * A_.hjiu[ij]);
    wlf = 0.5 * (w[ijk] + w[ijkw]);
    wrf = 0.5 * (w[ijkr] + w[ijkwr]);
    double dc2 = -2.0 * gama * vol * A_.hkiu[ij] *
                 (u[ijk] * A_.hkiu[ij] + va * A_.hkju[ij] + QDIV(wrf - wlf, rdkp, A_.r_rp[ij] * rdkp_[k - 1]));
    double udisf = QDIV(0.5 * (u[ijk] + u[ijks]), A_.dix[ij], A_.r_dix[ij]);
    double udinf = QDIV(0.5 * (u[ijk] + u[ijkn]), A_.dix[ijn], A_.r_dix[ijn]);
    double vdjwf = QDIV(0.5 * (v[ijkw] + v[ijknw]), A_.djp[ijw], A_.r_djp[ijw]);
    double vdjef = QDIV(0.5 * (v[ijk] + v[ijkn]), A_.djp[ij], A_.r_djp[ij]);
    double dc3 = gama * vol * A_.hiju[ij] *
                 (QDIV(di * (udinf - udisf), dj, A_.r_dju[ij]) + QDIV(dj * (vdjef - vdjwf), di, A_.r_diu[ij]));
    double diffc = dc1 + dc2 + dc3;
    // log-law wall stress (set_u_int_block.F:353-439)
    long kio = (iva == 1 ? A_.off_ki : A_.off_jk)[blockIdx.y];
    long ijo = b.off2 - A_.off2_lev1_base;
    double dist, tw_mean, ut_mean, yplus_mean, uloglaw, tw;
    if (wallsf && j == 2) {
        double *twa = A_.tw_s + kio;
        dist = 0.5 * A_.dju[ij];
        tw_mean = fabs(twa[ki]);
        ut_mean = sqrt(tw_mean / rhosf);
        yplus_mean = dist * ut_mean * rhosf / visc;
        if (yplus_mean > ylaminar) {
            uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
            tw = u[ijk] * tw_mean / uloglaw;
        } else {
            tw = visc * u[ijk] / dist;
        }
        tjisf = areasf * tw;
        twa[ki] = (st1 * (tw + twa[ki]) - st2 * tw) * stden;
    }
    if (wallnf && j == nj) {
        double *twa = A_.tw_n + kio;
        dist = 0.5 * A_.dju[ij];
        tw_mean = fabs(twa[ki]);
        ut_mean = sqrt(tw_mean / rhonf);
        yplus_mean = dist * ut_mean * rhonf / visc;
        if (yplus_mean > ylaminar) {
            uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
            tw = u[ijk] * tw_mean / uloglaw;
        } else {
            tw = visc * u[ijk] / dist;
        }
        tjinf = -areanf * tw;
        twa[ki] = (st1 * (-tw + twa[ki]) - st2 * (-tw)) * stden;
    }
    long ijl = ijo + (ij - o2);  // this cell's entry of the (i, j) wall arrays
    if (walllf && k == 2) {
        double *twa = A_.tw_l;
        dist = 0.5 * rdku;
        tw_mean = fabs(twa[ijl]);
        ut_mean = sqrt(tw_mean / rholf);
        yplus_mean = dist * ut_mean * rholf / visc;
        if (yplus_mean > ylaminar) {
            uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
            tw = u[ijk] * tw_mean / uloglaw;
        } else {
            tw = visc * u[ijk] / dist;
        }
        tkilf = areak * tw;
        twa[ijl] = (st1 * (tw + twa[ijl]) - st2 * tw) * stden;
    }
    if (wallrf && k == nk) {
        double *twa = A_.tw_r;
        dist = 0.5 * rdku;
        tw_mean = fabs(twa[ijl]);
        ut_mean = sqrt(tw_mean / rhorf);
        yplus_mean = dist * ut_mean * rhorf / visc;
        if (yplus_mean > ylaminar) {
            uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
            tw = u[ijk] * tw_mean / uloglaw;
        } else {
            tw = visc * u[ijk] / dist;
        }
        tkirf = -areak * tw;
        twa[ijl] = (st1 * (-tw + twa[ijl]) - st2 * (-tw)) * stden;
    }
    double h = conf + conc + diffc + tiief - tiiwf + tjinf - tjisf + tkirf - tkilf;
    if (A_.fb) h += A_.fb[ijk] * vol;  // body force per unit volume (off unless set)
    A_.u_int[ijk] = u[ijk] * (rhou / rhonp1u) +
                    dtime / (rhonp1u * vol) *
                        (1.5 * h - 0.5 * A_.hu[ijk] +
                         QDIV(0.5 * (A_.p[ijk] - A_.p[ijkw]) * vol, A_.diu[ij], A_.r_diu[ij]));
    A_.hu[ijk] = h;
    (void)nip1;
}

// code/set_w_int_block.F:95-458 (real i, j, k; k from kstart)
__global__ void __launch_bounds__(128) k_set_w_int(const BlkDev *__restrict__ blk, WIntArgs A_,
                                                   double dtime, int iststep, double visc,
                                                   double ylaminar, double kappa, double cwfun)
{
    if (A_.iststep) iststep = *A_.iststep;
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long ijk = decode_interior(b, q, i, j, k);
    int kstart = (b.bc[4] != LES_BCT_PERIODIC_D && b.bc[4] != LES_BCT_INTERFACE_D) ? 3 : 2;
    if (k < kstart) return;
    int nkp1 = b.n[2], ni = b.n[0] - 1, nj = b.n[1] - 1;
    long io = 1, jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    double st1 = iststep - 1, st2 = iststep - 2, stden = 1.0 / iststep;
    const double w_wall = 0.0;
    const double *u = A_.u, *v = A_.v, *w = A_.w, *rho = A_.rho, *gam = A_.gam;
    const double *dkp = A_.dkp + b.off1k, *dkw = A_.dkw + b.off1k;
    const double *const *M = A_.m;
#define G(a, ii, jj) M[a][IDX2(b, ii, jj)]
#ifdef LES_FAST_PHYS
#define GI(a, ii, jj) A_.r[a][IDX2(b, ii, jj)]
    const double *rdkp_ = A_.rdkp + b.off1k, *rdkw_ = A_.rdkw + b.off1k;
#endif
    double radp = G(MW_RP, i, j), radw = G(MW_RP, i - 1, j), rade = G(MW_RP, i + 1, j);
    double rads = G(MW_RP, i, j - 1), radn = G(MW_RP, i, j + 1);
    long ijkw = ijk - io, ijke = ijk + io, ijks = ijk - jo, ijkn = ijk + jo, ijkl = ijk - ko, ijkr = ijk + ko;
    long ijkwl = ijkw - ko, ijksl = ijks - ko, ijkel = ijke - ko, ijknl = ijkn - ko;
    double rhowf = 0.25 * (rho[ijk] + rho[ijkl] + rho[ijkw] + rho[ijkwl]);
    double rhoef = 0.25 * (rho[ijk] + rho[ijkl] + rho[ijke] + rho[ijkel]);
    double rhosf = 0.25 * (rho[ijk] + rho[ijkl] + rho[ijks] + rho[ijksl]);
    double rhonf = 0.25 * (rho[ijk] + rho[ijkl] + rho[ijkn] + rho[ijknl]);
    double rholf = rho[ijkl], rhorf = rho[ijk];
    double rhow = 0.5 * (rho[ijk] + rho[ijkl]);
    double rhonp1w = 0.5 * (A_.rhonp1[ijk] + A_.rhonp1[ijkl]);
    double gamwf = visc + .25 * (gam[ijk] + gam[ijkl] + gam[ijkw] + gam[ijkwl]) * rhowf;
    double gamef = visc + .25 * (gam[ijk] + gam[ijkl] + gam[ijke] + gam[ijkel]) * rhoef;
    double gamsf = visc + .25 * (gam[ijk] + gam[ijkl] + gam[ijks] + gam[ijksl]) * rhosf;
    double gamnf = visc + .25 * (gam[ijk] + gam[ijkl] + gam[ijkn] + gam[ijknl]) * rhonf;
    double gamlf = visc + gam[ijkl] * rholf;
    double gamrf = visc + gam[ijk] * rhorf;
    double areawf = G(MW_RDJU, i, j) * dkw[k - 1];
    double areaef = G(MW_RDJU, i + 1, j) * dkw[k - 1];
    double areasf = G(MW_RDIV, i, j) * dkw[k - 1];
    double areanf = G(MW_RDIV, i, j + 1) * dkw[k - 1];
    double areak = G(MW_DIDJP, i, j);
    double vol = G(MW_RDIDJP, i, j) * dkw[k - 1];
    double uwf = 0.5 * (u[ijk] + u[ijkl]);
    double uef = 0.5 * (u[ijke] + u[ijkel]);
    double vsf = 0.5 * (v[ijk] + v[ijkl]);
    double vnf = 0.5 * (v[ijkn] + v[ijknl]);
    double wlf = 0.5 * (w[ijk] + w[ijkl]);
    double wrf = 0.5 * (w[ijkr] + w[ijk]);
    double gwf = 0.5 * (w[ijk] + w[ijkw]) * uwf * rhowf * areawf;
    double gef = 0.5 * (w[ijk] + w[ijke]) * uef * rhoef * areaef;
    double gsf = 0.5 * (w[ijk] + w[ijks]) * vsf * rhosf * areasf;
    double gnf = 0.5 * (w[ijk] + w[ijkn]) * vnf * rhonf * areanf;
    double glf = wlf * wlf * rholf * areak;
    double grf = wrf * wrf * rhorf * areak;
    double conf = -(gef - gwf) - (gnf - gsf) - (grf - glf);
    double u_wc = 0.25 * (u[ijk] + u[ijke] + u[ijkl] + u[ijkel]);
    double v_wc = 0.25 * (v[ijk] + v[ijkn] + v[ijkl] + v[ijknl]);
    double conc = -vol * rhow * (w[ijk] * (u_wc * G(MW_HKIP, i, j) + v_wc * G(MW_HKJP, i, j)));
    double galwf = QDIV(gamwf * areawf, G(MW_DIU, i, j), GI(MW_DIU, i, j));
    double galef = QDIV(gamef * areaef, G(MW_DIU, i + 1, j), GI(MW_DIU, i + 1, j));
    double galsf = QDIV(gamsf * areasf, G(MW_DJV, i, j), GI(MW_DJV, i, j));
    double galnf = QDIV(gamnf * areanf, G(MW_DJV, i, j + 1), GI(MW_DJV, i, j + 1));
    double gallf = QDIV(gamlf * areak, (radp * dkp[k - 2]), GI(MW_RP, i, j) * rdkp_[k - 2]);
    double galrf = QDIV(gamrf * areak, (radp * dkp[k - 1]), GI(MW_RP, i, j) * rdkp_[k - 1]);
    double radwf = 0.5 * (radp + radw), radef = 0.5 * (radp + rade);
    double radsf = 0.5 * (radp + rads), radnf = 0.5 * (radp + radn);
    double ulf = 0.5 * (u[ijkl] + u[ijkel]), urf = 0.5 * (u[ijk] + u[ijke]);
    double vlf = 0.5 * (v[ijkl] + v[ijknl]), vrf = 0.5 * (v[ijk] + v[ijkn]);
    double wwf = 0.5 * (w[ijk] + w[ijkw]), wef = 0.5 * (w[ijk] + w[ijke]);
    double wsf = 0.5 * (w[ijk] + w[ijks]), wnf = 0.5 * (w[ijk] + w[ijkn]);
    double twf = galwf * radwf * (QDIV(w[ijk], radp, GI(MW_RP, i, j)) - QDIV(w[ijkw], radw, GI(MW_RP, i - 1, j)));
    double tef = galef * radef * (QDIV(w[ijke], rade, GI(MW_RP, i + 1, j)) - QDIV(w[ijk], radp, GI(MW_RP, i, j)));
    double tsf = galsf * (w[ijk] - w[ijks]);
    double tnf = galnf * (w[ijkn] - w[ijk]);
    double tlf = 2.0 * gallf * (w[ijk] - w[ijkl]);
    double trf = 2.0 * galrf * (w[ijkr] - w[ijk]);
    double cwf = gamwf * areawf * (QDIV(u[ijk] - u[ijkl], dkw[k - 1], rdkw_[k - 1]) / radwf - wwf * G(MW_HKIU, i, j));
    double cef = gamef * areaef *
                 (QDIV(u[ijke] - u[ijkel], dkw[k - 1], rdkw_[k - 1]) / radef - wef * G(MW_HKIU, i + 1, j));
    double csf = (j == 2) ? 0.0
                          : gamsf * areasf *
                                (QDIV(v[ijk] - v[ijkl], dkw[k - 1], rdkw_[k - 1]) / radsf - wsf * G(MW_HKJV, i, j));
    double cnf = gamnf * areanf *
                 (QDIV(v[ijkn] - v[ijknl], dkw[k - 1], rdkw_[k - 1]) / radnf - wnf * G(MW_HKJV, i, j + 1));
    double clf = 2.0 * gamlf * areak * (ulf * G(MW_HKIP, i, j) + vlf * G(MW_HKJP, i, j));
    double crf = 2.0 * gamrf * areak * (urf * G(MW_HKIP, i, j) + vrf * G(MW_HKJP, i, j));
    double dwdy = QDIV(wnf - wsf, G(MW_DJP, i, j), GI(MW_DJP, i, j));
    double dvdz = QDIV(vrf - vlf, (radp * dkw[k - 1]), GI(MW_RP, i, j) * rdkw_[k - 1]);
    double dwdx = QDIV(wef - wwf, G(MW_DIP, i, j), GI(MW_DIP, i, j));
    double dudz = QDIV(urf - ulf, (radp * dkw[k - 1]), GI(MW_RP, i, j) * rdkw_[k - 1]);
    double diffc1 = G(MW_HKIP, i, j) * (dwdx + dudz - w[ijk] * G(MW_HKIP, i, j)) * vol * gamrf;
    double diffc2 = G(MW_HKJP, i, j) * (dwdy + dvdz - w[ijk] * G(MW_HKJP, i, j)) * vol * gamrf;
    double diffc = diffc1 + diffc2;
    double tikwf = twf + cwf, tikef = tef + cef, tjksf = tsf + csf, tjknf = tnf + cnf;
    double tkklf = tlf + clf, tkkrf = trf + crf;
    double dist, tw_mean, ut_mean, yplus_mean, uloglaw, tw;
    long kj = A_.off_jk[blockIdx.y] + (k - 1) + (long)nkp1 * (j - 1);
    long kii = A_.off_ki[blockIdx.y] + (k - 1) + (long)nkp1 * (i - 1);
    if (b.bc[0] == LES_BCT_WALL_D && i == 2) {
        double *t_ = A_.tw_wfk;
        dist = 0.5 * G(MW_DIP, i, j);
        tw_mean = fabs(t_[kj]);
        ut_mean = sqrt(tw_mean / rhowf);
        yplus_mean = dist * ut_mean * rhowf / visc;
        if (yplus_mean > ylaminar) {
            uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
            tw = w[ijk] * tw_mean / uloglaw;
        } else {
            tw = visc * w[ijk] / dist;
        }
        tikwf = areawf * tw;
        t_[kj] = (st1 * (tw + t_[kj]) - st2 * tw) * stden;
    }
    if (b.bc[1] == LES_BCT_WALL_D && i == ni) {
        double *t_ = A_.tw_efk;
        dist = 0.5 * G(MW_DIP, i, j);
        tw_mean = fabs(t_[kj]);
        ut_mean = sqrt(tw_mean / rhoef);
        yplus_mean = dist * ut_mean * rhoef / visc;
        if (yplus_mean > ylaminar) {
            uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
            tw = w[ijk] * tw_mean / uloglaw;
        } else {
            tw = visc * w[ijk] / dist;
        }
        tikef = -areaef * tw;
        t_[kj] = (st1 * (-tw + t_[kj]) - st2 * (-tw)) * stden;
    }
    if (b.bc[2] == LES_BCT_WALL_D && j == 2) {
        double *t_ = A_.tw_sfk;
        dist = 0.5 * G(MW_DJP, i, j);
        tw_mean = fabs(t_[kii]);
        ut_mean = sqrt(tw_mean / rhosf);
        yplus_mean = dist * ut_mean * rhosf / visc;
        if (yplus_mean > ylaminar) {
            uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
            tw = w[ijk] * tw_mean / uloglaw;
        } else {
            tw = visc * (w[ijk] - w_wall) / dist;
        }
        tjksf = areasf * (tw - w_wall / 0.005 * visc);
        t_[kii] = (st1 * (tw + t_[kii]) - st2 * tw) * stden;
    }
    if (b.bc[3] == LES_BCT_WALL_D && j == nj) {
        double *t_ = A_.tw_nfk;
        dist = 0.5 * G(MW_DJP, i, j);
        tw_mean = fabs(t_[kii]);
        ut_mean = sqrt(tw_mean / rhonf);
        yplus_mean = dist * ut_mean * rhonf / visc;
        if (yplus_mean > ylaminar) {
            uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
            tw = w[ijk] * tw_mean / uloglaw;
        } else {
            tw = visc * (w[ijk] - w_wall) / dist;
        }
        tjknf = -areanf * (tw + w_wall / 0.015 * visc);
        t_[kii] = (st1 * (-tw + t_[kii]) - st2 * (-tw)) * stden;
    }
    double difff = tikef - tikwf + tjknf - tjksf + tkkrf - tkklf;
    double h = conf + conc + difff + diffc;
    if (A_.fb) h += A_.fb[ijk] * vol;  // body force per unit volume (off unless set)
    A_.w_int[ijk] = w[ijk] * (rhow / rhonp1w) +
                    dtime / (vol * rhonp1w) * (1.5 * h - 0.5 * A_.hw[ijk] + 0.5 * areak * (A_.p[ijk] - A_.p[ijkl]));
    A_.hw[ijk] = h;
#undef G
#ifdef GI
#undef GI
#endif
}

// ---------------------------------------------------------- scalar
// gamlam := visc / 0.72 everywhere (set_gamsc1_bc.F first loop)
__global__ void k_fill(double *__restrict__ a, double val, long n)
{
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        a[q] = val;
}

// Face cells of set_gamsc1_bc / set_sc1_bc: segment 0 = i sides over
// (j, k), 1 = j sides over (i, k), 2 = k sides over (i, j); interiors of
// the faces only, so no two threads touch the same ghost.  mode 0 =
// set_gamsc1_bc (gamsc1, gamlam and the interface gradients), mode 1 =
// set_sc1_bc on `f`.
__global__ void k_face_bc(const BlkDev *__restrict__ blk, int mode, double *__restrict__ f,
                          double *__restrict__ gam, double *__restrict__ gaml,
                          const double *__restrict__ sc1, const double *__restrict__ diu,
                          const double *__restrict__ djv, const double *__restrict__ rp,
                          const double *__restrict__ dkp, double *__restrict__ grad, long gstride,
                          int gm)
{
    const BlkDev b = blk[blockIdx.z];
    int seg = blockIdx.y;
    int nip1 = b.n[0], njp1 = b.n[1], nkp1 = b.n[2];
    int ni = nip1 - 1, nj = njp1 - 1, nk = nkp1 - 1;
    long jo = nip1, ko = (long)nip1 * njp1;
    int na, nb_;
    if (seg == 0) { na = nj - 1; nb_ = nk - 1; }
    else if (seg == 1) { na = ni - 1; nb_ = nk - 1; }
    else { na = ni - 1; nb_ = nj - 1; }
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)na * nb_) return;
    int a = (int)(q % na) + 2, c = (int)(q / na) + 2;
    long base = b.off3 - 1;  // 1-based index -> 0-based position
    double *G6 = grad + (long)blockIdx.z * 6 * gstride;
    long st[2];
    int sides[2];
    long ghost[2], inner[2], per[2];
    long gpos[2];
    double gval[2] = {0., 0.};
    if (seg == 0) {
        int j = a, k = c;
        long jk = jo * (j - 1) + ko * (k - 1);
        sides[0] = 0; sides[1] = 1;
        ghost[0] = 1 + jk; inner[0] = 2 + jk; per[0] = ni + jk;
        ghost[1] = nip1 + jk; inner[1] = nip1 - 1 + jk; per[1] = 2 + jk;
        if (mode == 0) {
            long d2 = IDX2(b, 3, j), d2e = IDX2(b, ni, j);
            gval[0] = (sc1[base + 3 + jk] - sc1[base + 2 + jk]) / diu[d2];
            gval[1] = (sc1[base + nip1 - 1 + jk] - sc1[base + nip1 - 2 + jk]) / diu[d2e];
            gpos[0] = 0 * gstride + (j - 1) + (long)gm * (k - 1);
            gpos[1] = 1 * gstride + (j - 1) + (long)gm * (k - 1);
        }
    } else if (seg == 1) {
        int i = a, k = c;
        long ik = i + ko * (k - 1);
        sides[0] = 2; sides[1] = 3;
        ghost[0] = ik; inner[0] = ik + jo; per[0] = ik + jo * (nj - 1);
        ghost[1] = ik + jo * (njp1 - 1); inner[1] = ik + jo * (njp1 - 2); per[1] = ik + jo;
        if (mode == 0) {
            gval[0] = (sc1[base + ik + 2 * jo] - sc1[base + ik + jo]) / djv[IDX2(b, i, 3)];
            gval[1] = (sc1[base + ik + jo * (njp1 - 2)] - sc1[base + ik + jo * (njp1 - 3)]) / djv[IDX2(b, i, nj)];
            gpos[0] = 2 * gstride + (i - 1) + (long)gm * (k - 1);
            gpos[1] = 3 * gstride + (i - 1) + (long)gm * (k - 1);
        }
    } else {
        int i = a, j = c;
        long ij = i + jo * (j - 1);
        sides[0] = 4; sides[1] = 5;
        ghost[0] = ij; inner[0] = ij + ko; per[0] = ij + ko * (nk - 1);
        ghost[1] = ij + ko * (nkp1 - 1); inner[1] = ij + ko * (nkp1 - 2); per[1] = ij + ko;
        if (mode == 0) {
            double r = rp[IDX2(b, i, j)];
            gval[0] = (sc1[base + ij + 2 * ko] - sc1[base + ij + ko]) / (r * dkp[b.off1k + 1]);
            gval[1] = (sc1[base + ij + ko * (nkp1 - 2)] - sc1[base + ij + ko * (nkp1 - 3)]) /
                      (r * dkp[b.off1k + nk - 2]);
            gpos[0] = 4 * gstride + (i - 1) + (long)gm * (j - 1);
            gpos[1] = 5 * gstride + (i - 1) + (long)gm * (j - 1);
        }
    }
    (void)st;
    for (int e = 0; e < 2; e++) {
        int t = b.bc[sides[e]];
        long gh = base + ghost[e], in = base + inner[e], pe = base + per[e];
        if (mode == 0) {
            G6[gpos[e]] = gval[e];
            if (t == LES_BCT_PERIODIC_D) gam[gh] = gam[pe];
            else if (t == LES_BCT_WALL_D) { gam[gh] = -gam[in]; gaml[gh] = -gaml[in]; }
            else if (t != LES_BCT_INTERFACE_D) gam[gh] = gam[in];
        } else {
            if (t == LES_BCT_PERIODIC_D) f[gh] = f[pe];
            else if (t != LES_BCT_INTERFACE_D && t != 4 /* FIXED */) f[gh] = f[in];
        }
    }
}

// one hyperplane i + j + k = s of set_sc1_block (see the header comment)
// One point of set_sc1_block.F:66-505.  sc1 is read through L2 (__ldcg):
// in the persistent sweep other CTAs update it between planes.
#define LDS(x) __ldcg(sc1r + (x))
__device__ __forceinline__ void sc1_cell(const BlkDev &b, int bi, int i, int j, int k,
                                         const Sc1Args &A_, double dtime)
{
    const double lambda = 4.0, small = 1.e-30;
    int nip1 = b.n[0];
    int ni = nip1 - 1, nj = b.n[1] - 1, nk = b.n[2] - 1;
    long io = 1, jo = nip1, ko = (long)nip1 * b.n[1];
    long ijk = b.off3 + (i - 1) + jo * (j - 1) + ko * (k - 1);
    long ijkw = ijk - io, ijke = ijk + io, ijks = ijk - jo, ijkn = ijk + jo, ijkl = ijk - ko, ijkr = ijk + ko;
    const double *sc1r = A_.sc1;
    const double *rho = A_.rho, *gs = A_.gamsc1, *gl = A_.gamlam;
    const double *dkp = A_.dkp + b.off1k, *dkw = A_.dkw + b.off1k;
#define G(a, ii, jj) A_.m[a][IDX2(b, ii, jj)]
    double rhowf = 0.5 * (rho[ijk] + rho[ijkw]);
    double rhoef = 0.5 * (rho[ijk] + rho[ijke]);
    double rhosf = 0.5 * (rho[ijk] + rho[ijks]);
    double rhonf = 0.5 * (rho[ijk] + rho[ijkn]);
    double rholf = 0.5 * (rho[ijk] + rho[ijkl]);
    double rhorf = 0.5 * (rho[ijk] + rho[ijkr]);
    double rhop = rho[ijk];
    double gamwf = 0.5 * (gs[ijk] + gs[ijkw]) * rhowf + 0.5 * (gl[ijk] + gl[ijkw]);
    double gamef = 0.5 * (gs[ijk] + gs[ijke]) * rhoef + 0.5 * (gl[ijk] + gl[ijke]);
    double gamsf = 0.5 * (gs[ijk] + gs[ijks]) * rhosf + 0.5 * (gl[ijk] + gl[ijks]);
    double gamnf = 0.5 * (gs[ijk] + gs[ijkn]) * rhonf + 0.5 * (gl[ijk] + gl[ijkn]);
    double gamlf = 0.5 * (gs[ijk] + gs[ijkl]) * rholf + 0.5 * (gl[ijk] + gl[ijkl]);
    double gamrf = 0.5 * (gs[ijk] + gs[ijkr]) * rhorf + 0.5 * (gl[ijk] + gl[ijkr]);
    double uwf = A_.u[ijk], uef = A_.u[ijke], vsf = A_.v[ijk], vnf = A_.v[ijkn];
    double wlf = A_.w[ijk], wrf = A_.w[ijkr];
#ifdef LES_FAST_PHYS
#define GI(a, ii, jj) A_.r[a][IDX2(b, ii, jj)]
    const double *rdkp_ = A_.rdkp + b.off1k;
#endif
    double dfdxwf = QDIV(LDS(ijk) - LDS(ijkw), G(MW_DIU, i, j), GI(MW_DIU, i, j));
    double dfdxef = QDIV(LDS(ijke) - LDS(ijk), G(MW_DIU, i + 1, j), GI(MW_DIU, i + 1, j));
    const long gst = A_.gstride;
    const double *GR = A_.grad;
    int gm = A_.gm;
    double dfdxwwf, dfdxeef, dfdyssf, dfdynnf, dfdzllf, dfdzrrf;
    if (i == 2) dfdxwwf = (b.bc[0] != LES_BCT_INTERFACE_D) ? dfdxwf
                          : GR[(long)(A_.link[bi * 6 + 0]) * 6 * gst + 1 * gst + (j - 1) + (long)gm * (k - 1)];
    else dfdxwwf = QDIV(LDS(ijkw) - LDS(ijkw - io), G(MW_DIU, i - 1, j), GI(MW_DIU, i - 1, j));
    if (i == ni) dfdxeef = (b.bc[1] != LES_BCT_INTERFACE_D) ? dfdxef
                           : GR[(long)(A_.link[bi * 6 + 1]) * 6 * gst + 0 * gst + (j - 1) + (long)gm * (k - 1)];
    else dfdxeef = QDIV(LDS(ijke + io) - LDS(ijke), G(MW_DIU, i + 2, j), GI(MW_DIU, i + 2, j));
    double dfdysf = QDIV(LDS(ijk) - LDS(ijks), G(MW_DJV, i, j), GI(MW_DJV, i, j));
    double dfdynf = QDIV(LDS(ijkn) - LDS(ijk), G(MW_DJV, i, j + 1), GI(MW_DJV, i, j + 1));
    if (j == 2) dfdyssf = (b.bc[2] != LES_BCT_INTERFACE_D) ? dfdysf
                          : GR[(long)(A_.link[bi * 6 + 2]) * 6 * gst + 3 * gst + (i - 1) + (long)gm * (k - 1)];
    else dfdyssf = QDIV(LDS(ijks) - LDS(ijks - jo), G(MW_DJV, i, j - 1), GI(MW_DJV, i, j - 1));
    if (j == nj) dfdynnf = (b.bc[3] != LES_BCT_INTERFACE_D) ? dfdynf
                           : GR[(long)(A_.link[bi * 6 + 3]) * 6 * gst + 2 * gst + (i - 1) + (long)gm * (k - 1)];
    else dfdynnf = QDIV(LDS(ijkn + jo) - LDS(ijkn), G(MW_DJV, i, j + 2), GI(MW_DJV, i, j + 2));
    double rpij = G(MW_RP, i, j);
#ifdef LES_FAST_PHYS
    const double rrpij = GI(MW_RP, i, j);
#endif
    double dfdzlf = QDIV(LDS(ijk) - LDS(ijkl), (rpij * dkp[k - 2]), rrpij * rdkp_[k - 2]);
    double dfdzrf = QDIV(LDS(ijkr) - LDS(ijk), (rpij * dkp[k - 1]), rrpij * rdkp_[k - 1]);
    if (k == 2) dfdzllf = (b.bc[4] != LES_BCT_INTERFACE_D) ? dfdzlf
                          : GR[(long)(A_.link[bi * 6 + 4]) * 6 * gst + 5 * gst + (i - 1) + (long)gm * (j - 1)];
    else dfdzllf = QDIV(LDS(ijkl) - LDS(ijkl - ko), (rpij * dkp[k - 3]), rrpij * rdkp_[k - 3]);
    if (k == nk) dfdzrrf = (b.bc[5] != LES_BCT_INTERFACE_D) ? dfdzrf
                           : GR[(long)(A_.link[bi * 6 + 5]) * 6 * gst + 4 * gst + (i - 1) + (long)gm * (j - 1)];
    else dfdzrrf = QDIV(LDS(ijkr + ko) - LDS(ijkr), (rpij * dkp[k]), rrpij * rdkp_[k]);
    double rwst = (uwf >= 0.0) ? (dfdxwwf + small) / (dfdxwf + small) : (dfdxef + small) / (dfdxwf + small);
    double rest = (uef > 0.0) ? (dfdxwf + small) / (dfdxef + small) : (dfdxeef + small) / (dfdxef + small);
    double rsth = (vsf >= 0.0) ? (dfdyssf + small) / (dfdysf + small) : (dfdynf + small) / (dfdysf + small);
    double rnth = (vnf > 0.0) ? (dfdysf + small) / (dfdynf + small) : (dfdynnf + small) / (dfdynf + small);
    double rlft = (wlf >= 0.0) ? (dfdzllf + small) / (dfdzlf + small) : (dfdzrf + small) / (dfdzlf + small);
    double rrht = (wrf > 0.0) ? (dfdzlf + small) / (dfdzrf + small) : (dfdzrrf + small) / (dfdzrf + small);
    double limw = fmax(0.0, fmin(lambda * rwst, 1.0));
    double lime = fmax(0.0, fmin(lambda * rest, 1.0));
    double lims = fmax(0.0, fmin(lambda * rsth, 1.0));
    double limn = fmax(0.0, fmin(lambda * rnth, 1.0));
    double liml = fmax(0.0, fmin(lambda * rlft, 1.0));
    double limr = fmax(0.0, fmin(lambda * rrht, 1.0));
    double s0 = LDS(ijk);
    double fwf, fef, fsf, fnf, flf, frf;
    if (uwf > 0.0) fwf = LDS(ijkw) + 0.5 * limw * (s0 - LDS(ijkw));
    else if (uwf < 0.0) fwf = s0 + 0.5 * limw * (LDS(ijkw) - s0);
    else fwf = 0.5 * (s0 + LDS(ijkw));
    if (uef > 0.0) fef = s0 + 0.5 * lime * (LDS(ijke) - s0);
    else if (uef < 0.0) fef = LDS(ijke) + 0.5 * lime * (s0 - LDS(ijke));
    else fef = 0.5 * (s0 + LDS(ijke));
    if (vsf > 0.0) fsf = LDS(ijks) + 0.5 * lims * (s0 - LDS(ijks));
    else if (vsf < 0.0) fsf = s0 + 0.5 * lims * (LDS(ijks) - s0);
    else fsf = 0.5 * (s0 + LDS(ijks));
    if (vnf > 0.0) fnf = s0 + 0.5 * limn * (LDS(ijkn) - s0);
    else if (vnf < 0.0) fnf = LDS(ijkn) + 0.5 * limn * (s0 - LDS(ijkn));
    else fnf = 0.5 * (s0 + LDS(ijkn));
    if (wlf > 0.0) flf = LDS(ijkl) + 0.5 * liml * (s0 - LDS(ijkl));
    else if (wlf < 0.0) flf = s0 + 0.5 * liml * (LDS(ijkl) - s0);
    else flf = 0.5 * (s0 + LDS(ijkl));
    if (wrf > 0.0) frf = s0 + 0.5 * limr * (LDS(ijkr) - s0);
    else if (wrf < 0.0) frf = LDS(ijkr) + 0.5 * limr * (s0 - LDS(ijkr));
    else frf = 0.5 * (s0 + LDS(ijkr));
    double areawf = G(MW_RDJU, i, j) * dkw[k - 1];
    double areaef = G(MW_RDJU, i + 1, j) * dkw[k - 1];
    double areasf = G(MW_RDIV, i, j) * dkw[k - 1];
    double areanf = G(MW_RDIV, i, j + 1) * dkw[k - 1];
    double areak = G(MW_DIDJP, i, j);
    double vol = G(MW_RDIDJP, i, j) * dkw[k - 1];
    double gwf = rhowf * uwf * fwf * areawf;
    double gef = rhoef * uef * fef * areaef;
    double gsf = rhosf * vsf * fsf * areasf;
    double gnf = rhonf * vnf * fnf * areanf;
    double glf = rholf * wlf * flf * areak;
    double grf = rhorf * wrf * frf * areak;
    double convf = -(gef - gwf) - (gnf - gsf) - (grf - glf);
    double twf = gamwf * areawf * dfdxwf;
    double tef = gamef * areaef * dfdxef;
    double tsf = gamsf * areasf * dfdysf;
    double tnf = gamnf * areanf * dfdynf;
    double tlf = gamlf * areak * dfdzlf;
    double trf = gamrf * areak * dfdzrf;
    double difff = (tef - twf) + (tnf - tsf) + (trf - tlf);
    double h = convf + difff;
    double tmp = s0 + dtime / (vol * rhop) * (1.5 * h - 0.5 * A_.hsc1[ijk]);
    A_.hsc1[ijk] = h;
    if (tmp < 0.0) tmp = 0.0;
    if (tmp > 1.0) tmp = 1.0;
    A_.sc1[ijk] = tmp;
#undef G
#ifdef GI
#undef GI
#endif
}
#undef LDS

__global__ void __launch_bounds__(128) k_sc1_wave(const BlkDev *__restrict__ blk, int s,
                                                  Sc1Args A_, double dtime)
{
    const BlkDev b = blk[blockIdx.y];
    int nj_ = b.n[1] - 2, nk_ = b.n[2] - 2;
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)nj_ * nk_) return;
    int k = (int)(q / nj_) + 2;
    int j = (int)(q - (long)(k - 2) * nj_) + 2;
    int i = s - j - k;
    if (i < 2 || i > b.n[0] - 1) return;
    sc1_cell(b, blockIdx.y, i, j, k, A_, dtime);
}

// Bounded grid barrier of the persistent sweep.  All CTAs of a cooperative
// launch are resident, so every arrival happens; the wait is still capped
// (limit polls, then err = 1 and every CTA leaves at its next barrier).
// Grid barrier of the persistent sweep, bounded.  Thread 0 of each CTA
// arrives with a release add on the counter (publishing the CTA's writes,
// which __syncthreads ordered before it) and polls the counter with
// acquire loads until all CTAs have arrived for this plane: one atomic and
// the polls on the critical path, no separate release flag or fences.
__device__ __forceinline__ bool wave_barrier(WaveSync *ws, unsigned nblk, unsigned target, long limit)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> count(ws->count);
        const unsigned goal = nblk * target;
        unsigned seen = count.fetch_add(1u, cuda::memory_order_release) + 1u;
        long it = 0;
        while (seen < goal) {
            if (*(volatile int *)&ws->err) {
                ok = 0;
                break;
            }
            if (++it > limit) {
                atomicExch(&ws->err, 1);
                ok = 0;
                break;
            }
            __nanosleep(32);
            seen = count.load(cuda::memory_order_acquire);
        }
    }
    __syncthreads();
    return ok != 0;
}

// One face of point (i, j, k) in set_sc1_block.F:66-505: axis d (0 x, 1 y,
// 2 z), hi = 0 for the low (W, S, L) face, 1 for the high (E, N, R) face.
// Every face runs the same code with axis-dependent indices, so the six
// faces of a point can go to six lanes without divergence.  Returns the
// convective flux g (rho u f area) and the diffusive flux t (gam area
// grad), with the reference's operands and order for each.
__device__ __forceinline__ void sc1_face(const BlkDev &b, int bi, int i, int j, int k, int d, int hi,
                                         const Sc1Args &A_, double &gout, double &tout)
{
    const double lambda = 4.0, small = 1.e-30;
    const double *sc1r = A_.sc1;
    const double *rho = A_.rho, *gs = A_.gamsc1, *gl = A_.gamlam;
    const double *dkp = A_.dkp + b.off1k, *dkw = A_.dkw + b.off1k;
#ifdef LES_FAST_PHYS
    const double *rdkp_ = A_.rdkp + b.off1k;
#endif
    const long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    const long ijk = b.off3 + (i - 1) + jo * (j - 1) + ko * (k - 1);
    const long sd = d == 0 ? 1 : d == 1 ? jo : ko;
    const int h = (d == 0 ? i : d == 1 ? j : k) + hi;  // high-side point of this face along d
    const int nd = d == 0 ? b.n[0] : d == 1 ? b.n[1] : b.n[2];
    const long ph = ijk + (hi ? sd : 0);
    const long pl = ph - sd;
    const long pn = hi ? ph : pl;          // the neighbour across the face
    // gradient across the face whose high-side point is hh (index phh)
    auto grad = [&](int hh, long phh) -> double {
        double df = __ldcg(sc1r + phh) - __ldcg(sc1r + phh - sd);
        if (d == 0) return QDIV(df, A_.m[MW_DIU][IDX2(b, hh, j)], A_.r[MW_DIU][IDX2(b, hh, j)]);
        if (d == 1) return QDIV(df, A_.m[MW_DJV][IDX2(b, i, hh)], A_.r[MW_DJV][IDX2(b, i, hh)]);
        return QDIV(df, (A_.m[MW_RP][IDX2(b, i, j)] * dkp[hh - 2]),
                    A_.r[MW_RP][IDX2(b, i, j)] * rdkp_[hh - 2]);
    };
    // interface gradient of the linked block (set_gamsc1_bc planes)
    auto igrad = [&](int side) -> double {
        long t = (d == 0) ? (j - 1) + (long)A_.gm * (k - 1)
                          : (d == 1) ? (i - 1) + (long)A_.gm * (k - 1) : (i - 1) + (long)A_.gm * (j - 1);
        return A_.grad[(long)A_.link[bi * 6 + side] * 6 * A_.gstride + (side ^ 1) * A_.gstride + t];
    };
    const double g0 = grad(h, ph);
    double gm, gp;
    if (h == 2) gm = (b.bc[2 * d] != LES_BCT_INTERFACE_D) ? g0 : igrad(2 * d);
    else gm = grad(h - 1, ph - sd);
    if (h == nd) gp = (b.bc[2 * d + 1] != LES_BCT_INTERFACE_D) ? g0 : igrad(2 * d + 1);
    else gp = grad(h + 1, ph + sd);
    const double *vel = d == 0 ? A_.u : d == 1 ? A_.v : A_.w;
    const double vf = vel[ph];
    // low faces test vel >= 0, high faces vel > 0 (the reference's rwst/rest)
    const bool up = hi ? (vf > 0.0) : (vf >= 0.0);
    const double r = up ? (gm + small) / (g0 + small) : (gp + small) / (g0 + small);
    const double lim = fmax(0.0, fmin(lambda * r, 1.0));
    const double s0 = __ldcg(sc1r + ijk), pa = __ldcg(sc1r + pl), pc = __ldcg(sc1r + ph);
    const double other = __ldcg(sc1r + pn);
    double f;
    if (vf > 0.0) f = pa + 0.5 * lim * (pc - pa);
    else if (vf < 0.0) f = pc + 0.5 * lim * (pa - pc);
    else f = 0.5 * (s0 + other);
    const double rhof = 0.5 * (rho[ijk] + rho[pn]);
    const double gamf = 0.5 * (gs[ijk] + gs[pn]) * rhof + 0.5 * (gl[ijk] + gl[pn]);
    double area;
    if (d == 0) area = A_.m[MW_RDJU][IDX2(b, h, j)] * dkw[k - 1];
    else if (d == 1) area = A_.m[MW_RDIV][IDX2(b, i, h)] * dkw[k - 1];
    else area = A_.m[MW_DIDJP][IDX2(b, i, j)];
    gout = rhof * vf * f * area;
    tout = gamf * area * g0;
}

// The whole in-place sweep in one cooperative launch.  Plane s holds the
// points with i + j + k = s; cum[s - smin][q] counts them over the (block,
// k) slices before q, so the points of a plane are enumerated densely.  A
// CTA takes 32 points at a time: warp w < 6 computes face w (W E S N L R) of
// all 32, warp 6 loads the point data, then combines the six faces in the
// reference's order and updates the points.  Every FP64 instruction thus
// runs with full warps (the FP64 pipe costs the same per warp instruction
// whatever the active mask).  A bounded grid barrier separates the planes.
// Results equal k_sc1_wave's.
__global__ void __launch_bounds__(256) k_sc1_sweep(const BlkDev *__restrict__ blk,
                                                   const int *__restrict__ cum,
                                                   const int2 *__restrict__ slice, int nslice,
                                                   int smin, int smax, Sc1Args A_, double dtime,
                                                   WaveSync *ws, long limit)
{
    extern __shared__ int scum[];
    __shared__ double fg[6][32], ft[6][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int s = smin; s <= smax; s++) {
        const int *row = cum + (long)(s - smin) * (nslice + 1);
        for (int q = threadIdx.x; q <= nslice; q += blockDim.x) scum[q] = row[q];
        __syncthreads();
        const int ncell = scum[nslice];
        for (long tb = (long)blockIdx.x * 32; tb < ncell; tb += (long)gridDim.x * 32) {
            const long t = tb + lane;
            const bool valid = t < ncell;
            int bi = 0, i = 0, j = 0, k = 0;
            if (valid) {
                int lo = 0, hi = nslice;
                while (hi - lo > 1) {
                    int mid = (lo + hi) >> 1;
                    if (scum[mid] <= t) lo = mid;
                    else hi = mid;
                }
                const int2 sl = slice[lo];
                bi = sl.x;
                k = sl.y;
                int jlo = s - k - (blk[bi].n[0] - 1);
                if (jlo < 2) jlo = 2;
                j = jlo + (int)(t - scum[lo]);
                i = s - j - k;
            }
            double s0 = 0., hold = 0., vr = 0.;
            long ijk = 0;
            if (w < 6) {
                if (valid) {
                    double gf, tf;
                    sc1_face(blk[bi], bi, i, j, k, w >> 1, w & 1, A_, gf, tf);
                    fg[w][lane] = gf;
                    ft[w][lane] = tf;
                }
            } else if (w == 6 && valid) {
                const BlkDev &b = blk[bi];
                ijk = b.off3 + (i - 1) + (long)b.n[0] * (j - 1) + (long)b.n[0] * b.n[1] * (k - 1);
                double vol = A_.m[MW_RDIDJP][IDX2(b, i, j)] * A_.dkw[b.off1k + k - 1];
                vr = dtime / (vol * A_.rho[ijk]);
                s0 = __ldcg(A_.sc1 + ijk);
                hold = A_.hsc1[ijk];
            }
            __syncthreads();
            if (w == 6 && valid) {
                double convf = -(fg[1][lane] - fg[0][lane]) - (fg[3][lane] - fg[2][lane]) -
                               (fg[5][lane] - fg[4][lane]);
                double difff = (ft[1][lane] - ft[0][lane]) + (ft[3][lane] - ft[2][lane]) +
                               (ft[5][lane] - ft[4][lane]);
                double hh = convf + difff;
                double tmp = s0 + vr * (1.5 * hh - 0.5 * hold);
                A_.hsc1[ijk] = hh;
                if (tmp < 0.0) tmp = 0.0;
                if (tmp > 1.0) tmp = 1.0;
                A_.sc1[ijk] = tmp;
            }
            __syncthreads();
        }
        if (!wave_barrier(ws, gridDim.x, (unsigned)(s - smin + 1), limit)) return;
    }
}

// code/set_sc1var_block.F:26-66
__global__ void k_sc1var(const BlkDev *__restrict__ blk, const double *__restrict__ sc1,
                         double *__restrict__ sc1var, const double *__restrict__ dip,
                         const double *__restrict__ djp, const double *__restrict__ rp,
                         const double *__restrict__ dkp, const double *__restrict__ dkw, SgsFast F)
{
    (void)F;
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long ijk = decode_interior(b, q, i, j, k);
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    const double cfv = 0.1;
    long ij = IDX2(b, i, j);
    double fwf = 0.5 * (sc1[ijk] + sc1[ijk - 1]);
    double fef = 0.5 * (sc1[ijk] + sc1[ijk + 1]);
    double fsf = 0.5 * (sc1[ijk] + sc1[ijk - jo]);
    double fnf = 0.5 * (sc1[ijk] + sc1[ijk + jo]);
    double flf = 0.5 * (sc1[ijk] + sc1[ijk - ko]);
    double frf = 0.5 * (sc1[ijk] + sc1[ijk + ko]);
    double dfdip = QDIV(fef - fwf, dip[ij], F.r_dip[ij]);
    double dfdjp = QDIV(fnf - fsf, djp[ij], F.r_djp[ij]);
    double dfdkp = QDIV(frf - flf, (rp[ij] * dkw[b.off1k + k - 1]), F.r_rp[ij] * F.r_dkw[b.off1k + k - 1]);
    double dfdijk = dfdip * dfdip + dfdjp * dfdjp + dfdkp * dfdkp;
#ifdef LES_FAST_PHYS
    double delta = F.delta2d[ij] * F.delta1d[b.off1k + k - 1];
#else
    double dk = rp[ij] * dkp[b.off1k + k - 1];
    double delta = pow(dip[ij] * djp[ij] * dk, .33333333);
#endif
    sc1var[ijk] = cfv * dfdijk * (delta * delta);
}

static inline unsigned nbk(long n, int t) { return (unsigned)((n + t - 1) / t); }

void launch_set_u_int(const BlkDev *blk, int nb, long maxcell, int iva, const UIntArgs &a,
                      double dtime, int iststep, double visc, double ylaminar, double kappa,
                      double cwfun, cudaStream_t st)
{
    k_set_u_int<<<dim3(nbk(maxcell, 128), nb), 128, 0, st>>>(blk, iva, a, dtime, iststep, visc, ylaminar,
                                                            kappa, cwfun);
    les::count_launch(1);
}

void launch_set_w_int(const BlkDev *blk, int nb, long maxcell, const WIntArgs &a, double dtime,
                      int iststep, double visc, double ylaminar, double kappa, double cwfun,
                      cudaStream_t st)
{
    k_set_w_int<<<dim3(nbk(maxcell, 128), nb), 128, 0, st>>>(blk, a, dtime, iststep, visc, ylaminar, kappa,
                                                            cwfun);
    les::count_launch(1);
}

void launch_fill(double *a, double val, long n, cudaStream_t st)
{
    unsigned g = nbk(n, 256);
    k_fill<<<g > 4096 ? 4096 : g, 256, 0, st>>>(a, val, n);
    les::count_launch(1);
}

void launch_face_bc(const BlkDev *blk, int nb, long maxface, int mode, double *f, double *gam,
                    double *gaml, const double *sc1, const double *diu, const double *djv,
                    const double *rp, const double *dkp, double *grad, long gstride, int gm,
                    cudaStream_t st)
{
    k_face_bc<<<dim3(nbk(maxface, 128), 3, nb), 128, 0, st>>>(blk, mode, f, gam, gaml, sc1, diu, djv, rp, dkp,
                                                             grad, gstride, gm);
    les::count_launch(1);
}

void launch_sc1_waves(const BlkDev *blk, int nb, long maxjk, int smin, int smax, const Sc1Args &a,
                      double dtime, cudaStream_t st)
{
    unsigned gx = nbk(maxjk, 128);
    for (int s = smin; s <= smax; s++) k_sc1_wave<<<dim3(gx, nb), 128, 0, st>>>(blk, s, a, dtime);
    les::count_launch(smax - smin + 1);
}

int sc1_sweep_max_ctas(int smem)
{
    int dev = 0, nsm = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sc1_sweep, 256, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    // three CTAs per SM: fewer arrivals per barrier against work per plane
    // (measured on the 256x192x128 mixing layer, FP32 physics: 1, 2, 3 per
    // SM gave 20.8, 18.7, 18.2 ms per step)
    return nsm * (per < 3 ? per : 3);
}

cudaError_t launch_sc1_sweep(const BlkDev *blk, const int *cum, const int2 *slice, int nslice, int nctas,
                             int smin, int smax, const Sc1Args &a, double dtime, WaveSync *ws, long limit,
                             cudaStream_t st)
{
    Sc1Args A = a;
    void *args[] = {(void *)&blk, (void *)&cum, (void *)&slice, (void *)&nslice, (void *)&smin,
                    (void *)&smax, (void *)&A, (void *)&dtime, (void *)&ws, (void *)&limit};
    size_t smem = sizeof(int) * (nslice + 1);
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_sc1_sweep, dim3(nctas), dim3(256), args, smem, st);
    les::count_launch(1);
    return e;
}

void launch_sc1var(const BlkDev *blk, int nb, long maxcell, const double *sc1, double *sc1var,
                   const double *dip, const double *djp, const double *rp, const double *dkp,
                   const double *dkw, const SgsFast &f, cudaStream_t st)
{
    k_sc1var<<<dim3(nbk(maxcell, 128), nb), 128, 0, st>>>(blk, sc1, sc1var, dip, djp, rp, dkp, dkw, f);
    les::count_launch(1);
}

} // namespace LES_PHYS_NS
