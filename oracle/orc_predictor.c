/*
 * orc_predictor.c -- oracle: Adams-Bashforth momentum predictor.
 * TEST INFRASTRUCTURE ONLY.
 *
 *   set_uv_int / set_u_int_block  code/set_uv_int.F:5-164,
 *                                 code/set_u_int_block.F:7-466
 *   set_w_int / set_w_int_block   code/set_w_int.F:5-141,
 *                                 code/set_w_int_block.F:9-463
 * The v component runs set_u_int_block with the i and j roles swapped
 * (code/step.F:319-326, set_uv_int.F:119-142).  Every cell writes only its
 * own u_int / hu entry and its own wall-stress entry, so the loop order does
 * not change the result; it is kept anyway.
 */
#include <math.h>
#include "orc_internal.h"

/* index of the metric table passed in m[] (comp_metric order) */
enum { M_DIP, M_DIU, M_DIV, M_DIX, M_RDIP, M_RDIV, M_RDIX, M_DJP, M_DJU, M_DJV, M_DJX, M_RDJP,
       M_RDJU, M_RDJX, M_HIJP, M_HJIP, M_HKIP, M_HKJP, M_HIJU, M_HJIU, M_HKIU, M_HKJU, M_HIJV,
       M_HJIV, M_HKIV, M_HKJV, M_RP, M_RU, M_RV, M_DIDJP, M_RDIDJP, M_DIDJU, M_RDIDJU, M_DJDIV,
       M_RDJDIV };

/* code/set_u_int_block.F:103-462, arguments as set_uv_int passes them */
static void set_u_int_block(int nip1, int njp1, int nkp1, long io, long jo, long ko, long io_ij,
                            long jo_ij, double dtime, const double *dip, const double *diu,
                            const double *dix, const double *rdix, const double *djp,
                            const double *dju, const double *djv, const double *djx,
                            const double *rdjp, const double *rdju, const double *didjp,
                            const double *didju, const double *rdidju, const double *hijp,
                            const double *hiju, const double *hjiu, const double *hkiu,
                            const double *hkju, const double *rp, const double *ru,
                            const double *dkp, const double *dkw, double *u_int, double *hu,
                            const double *u, const double *v, const double *w, const double *p,
                            const double *rho, const double *rhonp1, const double *gam,
                            double *tw_sfi, double *tw_nfi, double *tw_lfi, double *tw_rfi,
                            int wallwf, int wallef, int wallsf, int wallnf, int walllf,
                            int wallrf, int istart, int iststep, double visc, double ylaminar,
                            double kappa, double cwfun)
{
    (void)didjp;
    (void)wallwf;
    (void)wallef;
    int ni = nip1 - 1, nj = njp1 - 1, nk = nkp1 - 1;
    double st1 = iststep - 1, st2 = iststep - 2, stden = 1.0 / iststep;
    for (int j = 2; j <= nj; j++) {
        long joff = 1 + jo * (j - 1), joff_ij = 1 + jo_ij * (j - 1);
        for (int i = istart; i <= ni; i++) {
            long ijoff = io * (i - 1) + joff;
            long ij = io_ij * (i - 1) + joff_ij, ijw = ij - io_ij, ijs = ij - jo_ij;
            long ijn = ij + jo_ij, ijnw = ijw + jo_ij;
            long ioff_ki = (long)nkp1 * (i - 1);
            double di = A(diu, ij), dj = A(dju, ij);
            for (int k = 2; k <= nk; k++) {
                long ijk = ko * (k - 1) + ijoff, ki = k + ioff_ki;
                long ijkw = ijk - io, ijke = ijk + io, ijks = ijk - jo, ijkn = ijk + jo;
                long ijkl = ijk - ko, ijkr = ijk + ko;
                long ijksw = ijks - io, ijknw = ijkn - io, ijkwl = ijkw - ko, ijkwr = ijkw + ko;
                double rdkp = A(rp, ij) * A(dkp, k);
                double rdku = A(ru, ij) * A(dkp, k);
                double va = 0.25 * (A(v, ijk) + A(v, ijkn) + A(v, ijkw) + A(v, ijknw));
                double wa = 0.25 * (A(w, ijk) + A(w, ijkr) + A(w, ijkw) + A(w, ijkwr));
                double rhoa = 0.5 * (A(rho, ijkw) + A(rho, ijk));
                double gama = 0.5 * (A(gam, ijkw) + A(gam, ijk));
                double rhowf = A(rho, ijkw), rhoef = A(rho, ijk);
                double rhosf = 0.25 * (A(rho, ijk) + A(rho, ijkw) + A(rho, ijks) + A(rho, ijksw));
                double rhonf = 0.25 * (A(rho, ijk) + A(rho, ijkw) + A(rho, ijkn) + A(rho, ijknw));
                double rholf = 0.25 * (A(rho, ijk) + A(rho, ijkw) + A(rho, ijkl) + A(rho, ijkwl));
                double rhorf = 0.25 * (A(rho, ijk) + A(rho, ijkw) + A(rho, ijkr) + A(rho, ijkwr));
                double rhou = 0.5 * (A(rho, ijk) + A(rho, ijkw));
                double rhonp1u = 0.5 * (A(rhonp1, ijk) + A(rhonp1, ijkw));
                double gamwf = visc + A(gam, ijkw) * rhowf;
                double gamef = visc + A(gam, ijk) * rhoef;
                double gamsf = visc + .25 * (A(gam, ijk) + A(gam, ijkw) + A(gam, ijks) + A(gam, ijksw)) * rhosf;
                double gamnf = visc + .25 * (A(gam, ijk) + A(gam, ijkw) + A(gam, ijkn) + A(gam, ijknw)) * rhonf;
                double gamlf = visc + .25 * (A(gam, ijk) + A(gam, ijkw) + A(gam, ijkl) + A(gam, ijkwl)) * rholf;
                double gamrf = visc + .25 * (A(gam, ijk) + A(gam, ijkw) + A(gam, ijkr) + A(gam, ijkwr)) * rhorf;
                double areawf = A(rdjp, ijw) * A(dkp, k);
                double areaef = A(rdjp, ij) * A(dkp, k);
                double areasf = A(rdix, ij) * A(dkp, k);
                double areanf = A(rdix, ijn) * A(dkp, k);
                double areak = A(didju, ij);
                double vol = A(rdidju, ij) * A(dkp, k);
                double uwf = 0.5 * (A(u, ijk) + A(u, ijkw));
                double uef = 0.5 * (A(u, ijk) + A(u, ijke));
                double vsf = 0.5 * (A(v, ijk) + A(v, ijkw));
                double vnf = 0.5 * (A(v, ijkn) + A(v, ijknw));
                double wlf = 0.5 * (A(w, ijk) + A(w, ijkw));
                double wrf = 0.5 * (A(w, ijkr) + A(w, ijkwr));
                double gwf = uwf * uwf * rhowf * areawf;
                double gef = uef * uef * rhoef * areaef;
                double gsf = 0.5 * (A(u, ijk) + A(u, ijks)) * vsf * rhosf * areasf;
                double gnf = 0.5 * (A(u, ijk) + A(u, ijkn)) * vnf * rhonf * areanf;
                double glf = 0.5 * (A(u, ijk) + A(u, ijkl)) * wlf * rholf * areak;
                double grf = 0.5 * (A(u, ijk) + A(u, ijkr)) * wrf * rhorf * areak;
                double conf = -(gef - gwf) - (gnf - gsf) - (grf - glf);
                double cc1 = A(hjiu, ij) * rhoa * (va * va) * vol;
                double cc2 = A(hkiu, ij) * rhoa * (wa * wa) * vol;
                double cc3 = -A(hiju, ij) * rhoa * va * A(u, ijk) * vol;
                double conc = cc1 + cc2 + cc3;
                double galwf = gamwf * areawf / A(dip, ijw);
                double galef = gamef * areaef / A(dip, ij);
                double galsf = gamsf * areasf / A(djx, ij);
                double galnf = gamnf * areanf / A(djx, ijn);
                double gallf = gamlf * areak / (A(rp, ij) * A(dkw, k));
                double galrf = gamrf * areak / (A(rp, ij) * A(dkw, k + 1));
                double vwf = 0.5 * (A(v, ijkw) + A(v, ijknw));
                double vef = 0.5 * (A(v, ijk) + A(v, ijkn));
                double twf = galwf * 2.0 * (A(u, ijk) - A(u, ijkw));
                double tef = galef * 2.0 * (A(u, ijke) - A(u, ijk));
                double tsf = galsf * A(dix, ij) * (A(u, ijk) / A(diu, ij) - A(u, ijks) / A(diu, ijs));
                double tnf = galnf * A(dix, ijn) * (A(u, ijkn) / A(diu, ijn) - A(u, ijk) / A(diu, ij));
                double tlf = gallf * (A(u, ijk) - A(u, ijkl));
                double trf = galrf * (A(u, ijkr) - A(u, ijk));
                double cwf = 2.0 * gamwf * areawf * vwf * A(hijp, ijw);
                double cef = 2.0 * gamef * areaef * vef * A(hijp, ij);
                double csf = gamsf * areasf * A(djx, ij) * (A(v, ijk) / A(djv, ij) - A(v, ijkw) / A(djv, ijw)) /
                             A(dix, ij);
                double cnf = gamnf * areanf * A(djx, ijn) * (A(v, ijkn) / A(djv, ijn) - A(v, ijknw) / A(djv, ijnw)) /
                             A(dix, ijn);
                double clf = gamlf * areak * A(ru, ij) * (A(w, ijk) / A(rp, ij) - A(w, ijkw) / A(rp, ijw)) / A(diu, ij);
                double crf = gamrf * areak * A(ru, ij) * (A(w, ijkr) / A(rp, ij) - A(w, ijkwr) / A(rp, ijw)) / A(diu, ij);
                double tiiwf = twf + cwf, tiief = tef + cef, tjisf = tsf + csf, tjinf = tnf + cnf;
                double tkilf = tlf + clf, tkirf = trf + crf;
                vsf = 0.5 * (A(v, ijk) + A(v, ijkw));
                vnf = 0.5 * (A(v, ijkn) + A(v, ijknw));
                double dc1 = -2.0 * gama * vol * A(hjiu, ij) * ((vnf - vsf) / A(dju, ij) + A(u, ijk) * A(hjiu, ij));
                wlf = 0.5 * (A(w, ijk) + A(w, ijkw));
                wrf = 0.5 * (A(w, ijkr) + A(w, ijkwr));
                double dc2 = -2.0 * gama * vol * A(hkiu, ij) *
                             (A(u, ijk) * A(hkiu, ij) + va * A(hkju, ij) + (wrf - wlf) / rdkp);
                double udisf = 0.5 * (A(u, ijk) + A(u, ijks)) / A(dix, ij);
                double udinf = 0.5 * (A(u, ijk) + A(u, ijkn)) / A(dix, ijn);
                double vdjwf = 0.5 * (A(v, ijkw) + A(v, ijknw)) / A(djp, ijw);
                double vdjef = 0.5 * (A(v, ijk) + A(v, ijkn)) / A(djp, ij);
                double dc3 = gama * vol * A(hiju, ij) * (di * (udinf - udisf) / dj + dj * (vdjef - vdjwf) / di);
                double diffc = dc1 + dc2 + dc3;
                double dist, tw_mean, ut_mean, yplus_mean, uloglaw, tw;
                if (wallsf && j == 2) {
                    dist = 0.5 * A(dju, ij);
                    tw_mean = fabs(A(tw_sfi, ki));
                    ut_mean = sqrt(tw_mean / rhosf);
                    yplus_mean = dist * ut_mean * rhosf / visc;
                    if (yplus_mean > ylaminar) {
                        uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
                        tw = A(u, ijk) * tw_mean / uloglaw;
                    } else {
                        tw = visc * A(u, ijk) / dist;
                    }
                    tjisf = areasf * tw;
                    A(tw_sfi, ki) = (st1 * (tw + A(tw_sfi, ki)) - st2 * tw) * stden;
                }
                if (wallnf && j == nj) {
                    dist = 0.5 * A(dju, ij);
                    tw_mean = fabs(A(tw_nfi, ki));
                    ut_mean = sqrt(tw_mean / rhonf);
                    yplus_mean = dist * ut_mean * rhonf / visc;
                    if (yplus_mean > ylaminar) {
                        uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
                        tw = A(u, ijk) * tw_mean / uloglaw;
                    } else {
                        tw = visc * A(u, ijk) / dist;
                    }
                    tjinf = -areanf * tw;
                    A(tw_nfi, ki) = (st1 * (-tw + A(tw_nfi, ki)) - st2 * (-tw)) * stden;
                }
                if (walllf && k == 2) {
                    dist = 0.5 * rdku;
                    tw_mean = fabs(A(tw_lfi, ij));
                    ut_mean = sqrt(tw_mean / rholf);
                    yplus_mean = dist * ut_mean * rholf / visc;
                    if (yplus_mean > ylaminar) {
                        uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
                        tw = A(u, ijk) * tw_mean / uloglaw;
                    } else {
                        tw = visc * A(u, ijk) / dist;
                    }
                    tkilf = areak * tw;
                    A(tw_lfi, ij) = (st1 * (tw + A(tw_lfi, ij)) - st2 * tw) * stden;
                }
                if (wallrf && k == nk) {
                    dist = 0.5 * rdku;
                    tw_mean = fabs(A(tw_rfi, ij));
                    ut_mean = sqrt(tw_mean / rhorf);
                    yplus_mean = dist * ut_mean * rhorf / visc;
                    if (yplus_mean > ylaminar) {
                        uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
                        tw = A(u, ijk) * tw_mean / uloglaw;
                    } else {
                        tw = visc * A(u, ijk) / dist;
                    }
                    tkirf = -areak * tw;
                    A(tw_rfi, ij) = (st1 * (-tw + A(tw_rfi, ij)) - st2 * (-tw)) * stden;
                }
                double h = conf + conc + diffc + tiief - tiiwf + tjinf - tjisf + tkirf - tkilf;
                A(u_int, ijk) = A(u, ijk) * (rhou / rhonp1u) +
                                dtime / (rhonp1u * vol) *
                                    (1.5 * h - 0.5 * A(hu, ijk) + 0.5 * (A(p, ijk) - A(p, ijkw)) * vol / A(diu, ij));
                A(hu, ijk) = h;
            }
        }
    }
}

/* code/set_uv_int.F:63-160.  iva = 1 (u) or 2 (v).  metric[] holds the 35
 * comp_metric arrays (each tot2 long) in comp_metric order.  tw[4] are the
 * wall-stress arrays the calling routine passes for this component: for u
 * tw_sfi, tw_nfi (ki layout), tw_lfi, tw_rfi (ij layout); for v tw_wfj,
 * tw_efj (jk layout), tw_lfj, tw_rfj. */
void orc_set_uv_int(orc_ctx *c, int iva, double dtime, int iststep, double visc,
                    double ylaminar, double kappa, double cwfun, const double *u,
                    const double *v, const double *w, const double *p, const double *rho,
                    const double *rhonp1, const double *gam, double *u_int, double *hu,
                    const double *metric, const double *dkp, const double *dkw, double *tw_s,
                    double *tw_n, double *tw_l, double *tw_r)
{
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        long p3 = c->off3[1][b], p2 = c->off2[1][b], p1 = c->off1k[1][b];
        long pki = (iva == ORC_SV_U) ? c->offki[1][b] : c->offjk[1][b];
        const double *M[ORC_NMETRIC];
        for (int q = 0; q < ORC_NMETRIC; q++) M[q] = metric + (long)q * c->tot2 + p2;
        int d1 = (iva == ORC_SV_U) ? 1 : 2, d2 = (iva == ORC_SV_U) ? 2 : 1;
        int *bc = c->bl_bc[b];
        int walls[7];
        walls[2 * d1 - 1] = bc[2 * d1 - 2] == ORC_BCT_WALL;
        walls[2 * d1] = bc[2 * d1 - 1] == ORC_BCT_WALL;
        walls[2 * d2 - 1] = bc[2 * d2 - 2] == ORC_BCT_WALL;
        walls[2 * d2] = bc[2 * d2 - 1] == ORC_BCT_WALL;
        walls[5] = bc[4] == ORC_BCT_WALL;
        walls[6] = bc[5] == ORC_BCT_WALL;
        long ijko[4] = {0, 1, n[0], (long)n[0] * n[1]};
        long ijo[3] = {0, 1, n[0]};
        int nip1 = n[d1 - 1], njp1 = n[d2 - 1], nkp1 = n[2];
        long io = ijko[d1], jo = ijko[d2], ko = ijko[3];
        long io_ij = ijo[d1], jo_ij = ijo[d2];
        /* istart = nijkse(2*d1-1) with set_loop_bound(ivar = iva) */
        int s0 = bc[2 * d1 - 2];
        int istart = (s0 != ORC_BCT_PERIODIC && s0 != ORC_BCT_INTERFACE) ? 3 : 2;
        if (iva == ORC_SV_U)
            set_u_int_block(nip1, njp1, nkp1, io, jo, ko, io_ij, jo_ij, dtime, M[M_DIP], M[M_DIU],
                            M[M_DIX], M[M_RDIX], M[M_DJP], M[M_DJU], M[M_DJV], M[M_DJX], M[M_RDJP],
                            M[M_RDJU], M[M_DIDJP], M[M_DIDJU], M[M_RDIDJU], M[M_HIJP], M[M_HIJU],
                            M[M_HJIU], M[M_HKIU], M[M_HKJU], M[M_RP], M[M_RU], dkp + p1, dkw + p1,
                            u_int + p3, hu + p3, u + p3, v + p3, w + p3, p + p3, rho + p3,
                            rhonp1 + p3, gam + p3, tw_s + pki, tw_n + pki, tw_l + p2,
                            tw_r + p2, walls[1], walls[2], walls[3], walls[4],
                            walls[5], walls[6], istart, iststep, visc, ylaminar, kappa, cwfun);
        else
            set_u_int_block(nip1, njp1, nkp1, io, jo, ko, io_ij, jo_ij, dtime, M[M_DJP], M[M_DJV],
                            M[M_DJX], M[M_RDJX], M[M_DIP], M[M_DIV], M[M_DIU], M[M_DIX], M[M_RDIP],
                            M[M_RDIV], M[M_DIDJP], M[M_DJDIV], M[M_RDJDIV], M[M_HJIP], M[M_HJIV],
                            M[M_HIJV], M[M_HKJV], M[M_HKIV], M[M_RP], M[M_RV], dkp + p1, dkw + p1,
                            u_int + p3, hu + p3, u + p3, v + p3, w + p3, p + p3, rho + p3,
                            rhonp1 + p3, gam + p3, tw_s + pki, tw_n + pki, tw_l + p2,
                            tw_r + p2, walls[3], walls[4], walls[1], walls[2],
                            walls[5], walls[6], istart, iststep, visc, ylaminar, kappa, cwfun);
    }
    orc_swap_sc(c, 1, u_int, 2);
}

/* code/set_w_int_block.F:95-458 */
static void set_w_int_block(int nip1, int njp1, int nkp1, long io, long jo, long ko,
                            double dtime, double *const *M, const double *dkp,
                            const double *dkw, double *w_int, double *hw, const double *u,
                            const double *v, const double *w, const double *p,
                            const double *rho, const double *rhonp1, const double *gam,
                            double *tw_sfk, double *tw_nfk, double *tw_wfk, double *tw_efk,
                            int wallwf, int wallef, int wallsf, int wallnf, int kstart,
                            int iststep, double visc, double ylaminar, double kappa,
                            double cwfun)
{
    int ni = nip1 - 1, nj = njp1 - 1, nk = nkp1 - 1;
    double st1 = iststep - 1, st2 = iststep - 2, stden = 1.0 / iststep;
    double w_wall = 0.0; /* only ever assigned 0 (set_w_int_block.F:414,439) */
#define G(a, i, j) A2(M[a], i, j, nip1)
#define TWK(a, k, x) (a)[((long)(k) - 1) + (long)nkp1 * ((long)(x) - 1)]
    for (int j = 2; j <= nj; j++)
        for (int i = 2; i <= ni; i++) {
            double di = G(M_DIP, i, j), dj = G(M_DJP, i, j);
            double radp = G(M_RP, i, j), radw = G(M_RP, i - 1, j), rade = G(M_RP, i + 1, j);
            double rads = G(M_RP, i, j - 1), radn = G(M_RP, i, j + 1);
            (void)dj;
            (void)di;
            for (int k = kstart; k <= nk; k++) {
                long ijk = i + jo * (j - 1) + ko * (k - 1);
                long ijkw = ijk - io, ijke = ijk + io, ijks = ijk - jo, ijkn = ijk + jo;
                long ijkl = ijk - ko, ijkr = ijk + ko;
                long ijkwl = ijkw - ko, ijksl = ijks - ko, ijkel = ijke - ko, ijknl = ijkn - ko;
                double rhowf = 0.25 * (A(rho, ijk) + A(rho, ijkl) + A(rho, ijkw) + A(rho, ijkwl));
                double rhoef = 0.25 * (A(rho, ijk) + A(rho, ijkl) + A(rho, ijke) + A(rho, ijkel));
                double rhosf = 0.25 * (A(rho, ijk) + A(rho, ijkl) + A(rho, ijks) + A(rho, ijksl));
                double rhonf = 0.25 * (A(rho, ijk) + A(rho, ijkl) + A(rho, ijkn) + A(rho, ijknl));
                double rholf = A(rho, ijkl), rhorf = A(rho, ijk);
                double rhow = 0.5 * (A(rho, ijk) + A(rho, ijkl));
                double rhonp1w = 0.5 * (A(rhonp1, ijk) + A(rhonp1, ijkl));
                double gamwf = visc + .25 * (A(gam, ijk) + A(gam, ijkl) + A(gam, ijkw) + A(gam, ijkwl)) * rhowf;
                double gamef = visc + .25 * (A(gam, ijk) + A(gam, ijkl) + A(gam, ijke) + A(gam, ijkel)) * rhoef;
                double gamsf = visc + .25 * (A(gam, ijk) + A(gam, ijkl) + A(gam, ijks) + A(gam, ijksl)) * rhosf;
                double gamnf = visc + .25 * (A(gam, ijk) + A(gam, ijkl) + A(gam, ijkn) + A(gam, ijknl)) * rhonf;
                double gamlf = visc + A(gam, ijkl) * rholf;
                double gamrf = visc + A(gam, ijk) * rhorf;
                double areawf = G(M_RDJU, i, j) * A(dkw, k);
                double areaef = G(M_RDJU, i + 1, j) * A(dkw, k);
                double areasf = G(M_RDIV, i, j) * A(dkw, k);
                double areanf = G(M_RDIV, i, j + 1) * A(dkw, k);
                double areak = G(M_DIDJP, i, j);
                double vol = G(M_RDIDJP, i, j) * A(dkw, k);
                double uwf = 0.5 * (A(u, ijk) + A(u, ijkl));
                double uef = 0.5 * (A(u, ijke) + A(u, ijkel));
                double vsf = 0.5 * (A(v, ijk) + A(v, ijkl));
                double vnf = 0.5 * (A(v, ijkn) + A(v, ijknl));
                double wlf = 0.5 * (A(w, ijk) + A(w, ijkl));
                double wrf = 0.5 * (A(w, ijkr) + A(w, ijk));
                double gwf = 0.5 * (A(w, ijk) + A(w, ijkw)) * uwf * rhowf * areawf;
                double gef = 0.5 * (A(w, ijk) + A(w, ijke)) * uef * rhoef * areaef;
                double gsf = 0.5 * (A(w, ijk) + A(w, ijks)) * vsf * rhosf * areasf;
                double gnf = 0.5 * (A(w, ijk) + A(w, ijkn)) * vnf * rhonf * areanf;
                double glf = wlf * wlf * rholf * areak;
                double grf = wrf * wrf * rhorf * areak;
                double conf = -(gef - gwf) - (gnf - gsf) - (grf - glf);
                double u_wc = 0.25 * (A(u, ijk) + A(u, ijke) + A(u, ijkl) + A(u, ijkel));
                double v_wc = 0.25 * (A(v, ijk) + A(v, ijkn) + A(v, ijkl) + A(v, ijknl));
                double conc = -vol * rhow * (A(w, ijk) * (u_wc * G(M_HKIP, i, j) + v_wc * G(M_HKJP, i, j)));
                double galwf = gamwf * areawf / G(M_DIU, i, j);
                double galef = gamef * areaef / G(M_DIU, i + 1, j);
                double galsf = gamsf * areasf / G(M_DJV, i, j);
                double galnf = gamnf * areanf / G(M_DJV, i, j + 1);
                double gallf = gamlf * areak / (radp * A(dkp, k - 1));
                double galrf = gamrf * areak / (radp * A(dkp, k));
                double radwf = 0.5 * (radp + radw), radef = 0.5 * (radp + rade);
                double radsf = 0.5 * (radp + rads), radnf = 0.5 * (radp + radn);
                double ulf = 0.5 * (A(u, ijkl) + A(u, ijkel)), urf = 0.5 * (A(u, ijk) + A(u, ijke));
                double vlf = 0.5 * (A(v, ijkl) + A(v, ijknl)), vrf = 0.5 * (A(v, ijk) + A(v, ijkn));
                double wwf = 0.5 * (A(w, ijk) + A(w, ijkw)), wef = 0.5 * (A(w, ijk) + A(w, ijke));
                double wsf = 0.5 * (A(w, ijk) + A(w, ijks)), wnf = 0.5 * (A(w, ijk) + A(w, ijkn));
                double twf = galwf * radwf * (A(w, ijk) / radp - A(w, ijkw) / radw);
                double tef = galef * radef * (A(w, ijke) / rade - A(w, ijk) / radp);
                double tsf = galsf * (A(w, ijk) - A(w, ijks));
                double tnf = galnf * (A(w, ijkn) - A(w, ijk));
                double tlf = 2.0 * gallf * (A(w, ijk) - A(w, ijkl));
                double trf = 2.0 * galrf * (A(w, ijkr) - A(w, ijk));
                double cwf = gamwf * areawf * ((A(u, ijk) - A(u, ijkl)) / A(dkw, k) / radwf - wwf * G(M_HKIU, i, j));
                double cef = gamef * areaef * ((A(u, ijke) - A(u, ijkel)) / A(dkw, k) / radef - wef * G(M_HKIU, i + 1, j));
                double csf;
                if (j == 2)
                    csf = 0.0;
                else
                    csf = gamsf * areasf * ((A(v, ijk) - A(v, ijkl)) / A(dkw, k) / radsf - wsf * G(M_HKJV, i, j));
                double cnf = gamnf * areanf * ((A(v, ijkn) - A(v, ijknl)) / A(dkw, k) / radnf - wnf * G(M_HKJV, i, j + 1));
                double clf = 2.0 * gamlf * areak * (ulf * G(M_HKIP, i, j) + vlf * G(M_HKJP, i, j));
                double crf = 2.0 * gamrf * areak * (urf * G(M_HKIP, i, j) + vrf * G(M_HKJP, i, j));
                double dwdy = (wnf - wsf) / G(M_DJP, i, j);
                double dvdz = (vrf - vlf) / (radp * A(dkw, k));
                double dwdx = (wef - wwf) / G(M_DIP, i, j);
                double dudz = (urf - ulf) / (radp * A(dkw, k));
                double diffc1 = G(M_HKIP, i, j) * (dwdx + dudz - A(w, ijk) * G(M_HKIP, i, j)) * vol * gamrf;
                double diffc2 = G(M_HKJP, i, j) * (dwdy + dvdz - A(w, ijk) * G(M_HKJP, i, j)) * vol * gamrf;
                double diffc = diffc1 + diffc2;
                double tikwf = twf + cwf, tikef = tef + cef, tjksf = tsf + csf, tjknf = tnf + cnf;
                double tkklf = tlf + clf, tkkrf = trf + crf;
                double dist, tw_mean, ut_mean, yplus_mean, uloglaw, tw;
                if (wallwf && i == 2) {
                    dist = 0.5 * G(M_DIP, i, j);
                    tw_mean = fabs(TWK(tw_wfk, k, j));
                    ut_mean = sqrt(tw_mean / rhowf);
                    yplus_mean = dist * ut_mean * rhowf / visc;
                    if (yplus_mean > ylaminar) {
                        uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
                        tw = A(w, ijk) * tw_mean / uloglaw;
                    } else {
                        tw = visc * A(w, ijk) / dist;
                    }
                    tikwf = areawf * tw;
                    TWK(tw_wfk, k, j) = (st1 * (tw + TWK(tw_wfk, k, j)) - st2 * tw) * stden;
                }
                if (wallef && i == ni) {
                    dist = 0.5 * G(M_DIP, i, j);
                    tw_mean = fabs(TWK(tw_efk, k, j));
                    ut_mean = sqrt(tw_mean / rhoef);
                    yplus_mean = dist * ut_mean * rhoef / visc;
                    if (yplus_mean > ylaminar) {
                        uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
                        tw = A(w, ijk) * tw_mean / uloglaw;
                    } else {
                        tw = visc * A(w, ijk) / dist;
                    }
                    tikef = -areaef * tw;
                    TWK(tw_efk, k, j) = (st1 * (-tw + TWK(tw_efk, k, j)) - st2 * (-tw)) * stden;
                }
                if (wallsf && j == 2) {
                    dist = 0.5 * G(M_DJP, i, j);
                    tw_mean = fabs(TWK(tw_sfk, k, i));
                    ut_mean = sqrt(tw_mean / rhosf);
                    yplus_mean = dist * ut_mean * rhosf / visc;
                    if (yplus_mean > ylaminar) {
                        uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
                        tw = A(w, ijk) * tw_mean / uloglaw;
                    } else {
                        tw = visc * (A(w, ijk) - w_wall) / dist;
                    }
                    tjksf = areasf * (tw - w_wall / 0.005 * visc);
                    TWK(tw_sfk, k, i) = (st1 * (tw + TWK(tw_sfk, k, i)) - st2 * tw) * stden;
                }
                if (wallnf && j == nj) {
                    dist = 0.5 * G(M_DJP, i, j);
                    tw_mean = fabs(TWK(tw_nfk, k, i));
                    ut_mean = sqrt(tw_mean / rhonf);
                    yplus_mean = dist * ut_mean * rhonf / visc;
                    if (yplus_mean > ylaminar) {
                        uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
                        tw = A(w, ijk) * tw_mean / uloglaw;
                    } else {
                        tw = visc * (A(w, ijk) - w_wall) / dist;
                    }
                    tjknf = -areanf * (tw + w_wall / 0.015 * visc);
                    TWK(tw_nfk, k, i) = (st1 * (-tw + TWK(tw_nfk, k, i)) - st2 * (-tw)) * stden;
                }
                double difff = tikef - tikwf + tjknf - tjksf + tkkrf - tkklf;
                double h = conf + conc + difff + diffc;
                A(w_int, ijk) = A(w, ijk) * (rhow / rhonp1w) +
                                dtime / (vol * rhonp1w) * (1.5 * h - 0.5 * A(hw, ijk) + 0.5 * areak * (A(p, ijk) - A(p, ijkl)));
                A(hw, ijk) = h;
            }
        }
#undef G
#undef TWK
}

/* code/set_w_int.F:57-131.  tw_sfk, tw_nfk in (k, i) layout, tw_wfk,
 * tw_efk in (k, j) layout, level-1 ki / jk offsets. */
void orc_set_w_int(orc_ctx *c, double dtime, int iststep, double visc, double ylaminar,
                   double kappa, double cwfun, const double *u, const double *v,
                   const double *w, const double *p, const double *rho, const double *rhonp1,
                   const double *gam, double *w_int, double *hw, const double *metric,
                   const double *dkp, const double *dkw, double *tw_sfk, double *tw_nfk,
                   double *tw_wfk, double *tw_efk)
{
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        long p3 = c->off3[1][b], p2 = c->off2[1][b], p1 = c->off1k[1][b];
        double *M[ORC_NMETRIC];
        for (int q = 0; q < ORC_NMETRIC; q++) M[q] = (double *)metric + (long)q * c->tot2 + p2;
        int *bc = c->bl_bc[b];
        int kstart = (bc[4] != ORC_BCT_PERIODIC && bc[4] != ORC_BCT_INTERFACE) ? 3 : 2;
        set_w_int_block(n[0], n[1], n[2], 1, n[0], (long)n[0] * n[1], dtime, M, dkp + p1, dkw + p1,
                        w_int + p3, hw + p3, u + p3, v + p3, w + p3, p + p3, rho + p3, rhonp1 + p3,
                        gam + p3, tw_sfk + c->offki[1][b], tw_nfk + c->offki[1][b],
                        tw_wfk + c->offjk[1][b], tw_efk + c->offjk[1][b], bc[0] == ORC_BCT_WALL,
                        bc[1] == ORC_BCT_WALL, bc[2] == ORC_BCT_WALL, bc[3] == ORC_BCT_WALL, kstart,
                        iststep, visc, ylaminar, kappa, cwfun);
    }
    orc_swap_sc(c, 1, w_int, 2);
}
