/*
 * orc_sgs.c -- oracle: eddy-viscosity models.  TEST INFRASTRUCTURE ONLY.
 *
 * Restates subgrid (code/subgrid.F:5-107) with its Smagorinsky
 * (code/subgrid_smagorinsky.F:7-241), WALE (code/subgrid_wale.F:5-245) and
 * no-model branches, followed by the swaps of gam and gamsc1.
 * Fortran `x**2` with an integer exponent is x*x; a real exponent is pow().
 * The literal 0.33333333 is the reference's own (not 1/3).
 */
#include <math.h>
#include "orc_internal.h"

static void sgs_block(int model, double csles, int gotrad, double alpha, int nip1, int njp1,
                      int nkp1, double *gam, double *gamsc1, const double *u,
                      const double *v, const double *w, const double *sc1,
                      double *sc1var, double *sc1dis, const double *vdd,
                      const double *dip, const double *diu, const double *djp,
                      const double *djv, const double *dkp, const double *dkw,
                      const double *hijp, const double *hjip,
                      const double *hkip, const double *hkjp, const double *rp)
{
    const double sct = 0.3, cfv = 0.1;
    long jo = nip1, ko = (long)nip1 * njp1;
    int ni = nip1 - 1, nj = njp1 - 1, nk = nkp1 - 1;
    double onethird = 1.0 / 3.0;
#define G(a, i, j) A2(a, i, j, nip1)
    for (int k = 2; k <= nk; k++) {
        long koff = ko * (k - 1);
        for (int j = 2; j <= nj; j++) {
            long jk = jo * (j - 1) + koff;
            for (int i = 2; i <= ni; i++) {
                long ijk = i + jk;
                long ijkw = ijk - 1, ijke = ijk + 1, ijks = ijk - jo, ijkn = ijk + jo;
                long ijkl = ijk - ko, ijkr = ijk + ko;
                long ijkse = ijks + 1, ijknw = ijkn - 1, ijkne = ijkn + 1;
                long ijkel = ijke - ko, ijknl = ijkn - ko, ijkwr = ijkw + ko;
                long ijker = ijke + ko, ijksr = ijks + ko, ijknr = ijkn + ko;

                double fwf = 0.5 * (A(sc1, ijk) + A(sc1, ijkw));
                double fef = 0.5 * (A(sc1, ijk) + A(sc1, ijke));
                double fsf = 0.5 * (A(sc1, ijk) + A(sc1, ijks));
                double fnf = 0.5 * (A(sc1, ijk) + A(sc1, ijkn));
                double flf = 0.5 * (A(sc1, ijk) + A(sc1, ijkl));
                double frf = 0.5 * (A(sc1, ijk) + A(sc1, ijkr));
                double dfdip = (fef - fwf) / G(dip, i, j);
                double dfdjp = (fnf - fsf) / G(djp, i, j);
                double dfdkp = (frf - flf) / (G(rp, i, j) * A(dkw, k));

                double up = 0.5 * (A(u, ijk) + A(u, ijke));
                double vp = 0.5 * (A(v, ijk) + A(v, ijkn));
                double di = G(dip, i, j), dj = G(djp, i, j), dk;
                double vwf = 0.25 * (A(v, ijk) + A(v, ijkn) + A(v, ijkw) + A(v, ijknw));
                double vef = 0.25 * (A(v, ijk) + A(v, ijkn) + A(v, ijke) + A(v, ijkne));
                double usf = 0.25 * (A(u, ijk) + A(u, ijke) + A(u, ijks) + A(u, ijkse));
                double unf = 0.25 * (A(u, ijk) + A(u, ijke) + A(u, ijkn) + A(u, ijkne));
                double ulf = 0.25 * (A(u, ijk) + A(u, ijke) + A(u, ijkl) + A(u, ijkel));
                double urf = 0.25 * (A(u, ijk) + A(u, ijke) + A(u, ijkr) + A(u, ijker));
                double vlf = 0.25 * (A(v, ijk) + A(v, ijkn) + A(v, ijkl) + A(v, ijknl));
                double vrf = 0.25 * (A(v, ijk) + A(v, ijkn) + A(v, ijkr) + A(v, ijknr));

                double dudi = (A(u, ijke) - A(u, ijk)) / di + vp * G(hijp, i, j);
                double dvdi = (vef - vwf) / di - up * G(hijp, i, j);
                double dudj = (unf - usf) / dj - vp * G(hjip, i, j);
                double dvdj = (A(v, ijkn) - A(v, ijk)) / dj + up * G(hjip, i, j);
                double dwdi, dwdj, dudk, dvdk, dwdk;
                if (gotrad) {
                    double radp = G(rp, i, j), radw = G(rp, i - 1, j), rade = G(rp, i + 1, j);
                    double rads = G(rp, i, j - 1), radn = G(rp, i, j + 1);
                    dk = radp * A(dkp, k);
                    double hki = G(hkip, i, j), hkj = G(hkjp, i, j);
                    double wdrw = 0.5 * (A(w, ijkw) + A(w, ijkwr)) / radw;
                    double wdre = 0.5 * (A(w, ijke) + A(w, ijker)) / rade;
                    double wdrs = 0.5 * (A(w, ijks) + A(w, ijksr)) / rads;
                    double wdrn = 0.5 * (A(w, ijkn) + A(w, ijknr)) / radn;
                    dwdi = radp * (wdre - wdrw) / (G(diu, i, j) + G(diu, i + 1, j));
                    dwdj = radp * (wdrn - wdrs) / (G(djv, i, j) + G(djv, i, j + 1));
                    double wp = 0.5 * (A(w, ijk) + A(w, ijkr));
                    dudk = (urf - ulf) / dk - wp * hki;
                    dvdk = (vrf - vlf) / dk - wp * hkj;
                    dwdk = (A(w, ijkr) - A(w, ijk)) / dk + up * hki + vp * hkj;
                } else {
                    dk = A(dkp, k);
                    double wwf = 0.25 * (A(w, ijk) + A(w, ijkr) + A(w, ijkw) + A(w, ijkwr));
                    double wef = 0.25 * (A(w, ijk) + A(w, ijkr) + A(w, ijke) + A(w, ijker));
                    double wsf = 0.25 * (A(w, ijk) + A(w, ijkr) + A(w, ijks) + A(w, ijksr));
                    double wnf = 0.25 * (A(w, ijk) + A(w, ijkr) + A(w, ijkn) + A(w, ijknr));
                    dwdi = (wef - wwf) / di;
                    dwdj = (wnf - wsf) / dj;
                    dudk = (urf - ulf) / dk;
                    dvdk = (vrf - vlf) / dk;
                    dwdk = (A(w, ijkr) - A(w, ijk)) / dk;
                }
                double sijsij = dvdj * dvdj + dwdk * dwdk + dudi * dudi +
                                0.5 * ((dudj + dvdi) * (dudj + dvdi) + (dvdk + dwdj) * (dvdk + dwdj) +
                                       (dudk + dwdi) * (dudk + dwdi));
                double delta_xyz = pow(di * dj * dk, .33333333);
                double g;
                if (model == 1) {
                    /* subgrid_smagorinsky.F:215-222 */
                    double evisc = csles * delta_xyz * A(vdd, ijk);
                    evisc = evisc * evisc * sqrt(2.0 * sijsij);
                    g = evisc;
                } else if (model == 3) {
                    /* edge/subgrid_sigma.F:202-269; sqrt of the COMMON alpha
                       (cb.control.inc) as written there */
                    const double pi = 3.1415927;
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
                    double invari1 = g11 + g22 + g33;
                    double invari2 = 0.5 * (invari1 * invari1 - tracegg);
                    double invari3 = g11 * (g22 * g33 - g23 * g32) - g12 * (g21 * g33 - g23 * g31) +
                                     g13 * (g21 * g32 - g22 * g31);
                    double alpha1 = (invari1 * invari1 * 0.11111111) - (invari2 * onethird);
                    double alpha2 = (invari1 * invari1 * invari1 * 0.03703703703) -
                                    (invari1 * invari2 * 0.16666666666) + (invari3 * 0.5);
                    double alpha3 = onethird * acos(alpha2 / pow(alpha1, 1.5));
                    double invari13rd = invari1 * onethird;
                    double sqrtalpha = sqrt(alpha);
                    double sigma1 = pow(invari13rd + 2.0 * sqrtalpha * cos(alpha3), 0.5);
                    double sigma2 = pow(invari13rd - 2.0 * sqrtalpha * cos(pi * onethird + alpha3), 0.5);
                    double sigma3 = pow(invari13rd - 2.0 * sqrtalpha * cos(pi * onethird - alpha3), 0.5);
                    double sigmafinal = (sigma3 * (sigma1 - sigma2) * (sigma2 - sigma3)) / pow(sigma1, 2.0);
                    double evisc = (csles * delta_xyz) * (csles * delta_xyz);
                    g = evisc * sigmafinal;
                } else {
                    /* subgrid_wale.F:200-227 */
                    double g11 = dudi * dudi + dudj * dvdi + dudk * dwdi;
                    double g22 = dvdi * dudj + dvdj * dvdj + dvdk * dwdj;
                    double g33 = dwdi * dudk + dwdj * dvdk + dwdk * dwdk;
                    double g12 = dudi * dudj + dudj * dvdj + dudk * dwdj;
                    double g13 = dudi * dudk + dudj * dvdk + dudk * dwdk;
                    double g21 = dvdi * dudi + dvdj * dvdi + dvdk * dwdi;
                    double g23 = dvdi * dudk + dvdj * dvdk + dvdk * dwdk;
                    double g31 = dwdi * dudi + dwdj * dvdi + dwdk * dwdi;
                    double g32 = dwdi * dudj + dwdj * dvdj + dwdk * dwdj;
                    double tracet = onethird * (g11 + g22 + g33);
                    double sdij = (g11 - tracet) + (g22 - tracet) + (g33 - tracet) +
                                  0.5 * (g12 + g21) + 0.5 * (g13 + g31) + 0.5 * (g23 + g32);
                    double sd2 = sdij * sdij;
                    double ev = (csles * delta_xyz) * (csles * delta_xyz);
                    g = ev * (pow(sd2, 1.5) / (pow(sijsij, 2.5) + pow(sd2, 1.25)));
                }
                A(gam, ijk) = g;
                if (csles == 0.0)
                    A(gamsc1, ijk) = 0.0;
                else
                    A(gamsc1, ijk) = A(gam, ijk) / sct;
                double dfdijk = dfdip * dfdip + dfdjp * dfdjp + dfdkp * dfdkp;
                A(sc1var, ijk) = cfv * dfdijk * (delta_xyz * delta_xyz);
                A(sc1dis, ijk) = A(sc1var, ijk) * sqrt(2.0 * sijsij);
            }
        }
    }
#undef G
}

void orc_subgrid(orc_ctx *c, int model, double csles, int gotrad, double alpha,
                 double *gam, double *gamsc1, const double *u,
                 const double *v, const double *w, const double *sc1,
                 double *sc1var, double *sc1dis, const double *vd_damping,
                 const double *dip, const double *diu, const double *djp,
                 const double *djv, const double *dkp, const double *dkw,
                 const double *hijp, const double *hjip, const double *hkip,
                 const double *hkjp, const double *rp)
{
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        long p3 = c->off3[1][b], p2 = c->off2[1][b], p1 = c->off1k[1][b];
        if (model == 0) {
            /* subgrid_nosgs: gam = gamsc1 = 0.  Its sc1var uses a delta_xyz
             * that subgrid_nosgs.F never assigns; here it is taken as 0. */
            int *m = n;
            long jo = m[0], ko = (long)m[0] * m[1];
            for (int k = 2; k <= m[2] - 1; k++)
                for (int j = 2; j <= m[1] - 1; j++)
                    for (int i = 2; i <= m[0] - 1; i++) {
                        long q = p3 + i + jo * (j - 1) + ko * (k - 1);
                        A(gam, q) = 0.0;
                        A(gamsc1, q) = 0.0;
                        A(sc1var, q) = 0.0;
                        A(sc1dis, q) = 0.0;
                    }
        } else if (model >= 1 && model <= 3)
            sgs_block(model, csles, gotrad, alpha, n[0], n[1], n[2], gam + p3, gamsc1 + p3,
                      u + p3, v + p3, w + p3, sc1 + p3, sc1var + p3, sc1dis + p3,
                      vd_damping + p3, dip + p2, diu + p2, djp + p2, djv + p2,
                      dkp + p1, dkw + p1, hijp + p2, hjip + p2, hkip + p2,
                      hkjp + p2, rp + p2);
    }
    orc_swap_sc(c, 1, gam, 2);
    orc_swap_sc(c, 1, gamsc1, 2);
}
