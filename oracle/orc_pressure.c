/*
 * orc_pressure.c -- oracle: pressure equation assembly, multigrid solve,
 * pressure post-processing and the projection.  TEST INFRASTRUCTURE ONLY.
 *
 * Restates, one rank, FP64, in the reference's loop order:
 *   coeff_p / coeff_p_block        code/coeff_p.F:5-78, coeff_p_block.F:5-232
 *   sour_p / sour_p_block          code/sour_p.F:6-74, sour_p_block.F:5-170
 *   norms / norms_block            code/norms.F:5-127, norms_block.F:5-67
 *   sporlx / spor                  code/sporlx.F:5-276
 *   smooth                         code/smooth.F:5-105
 *   solversc                       code/solversc.F:7-48
 *   restriction / rest_block       code/restriction.F:5-68, rest_block.F:6-79
 *   prolongation / prol_block      code/prolongation.F:5-75, prol_block.F:10-250
 *   init_array                     code/init_array.F:5-77
 *   lmg_solve                      code/lmg_solve.F:5-172
 *   extrap_p / extrap_p_block      code/extrap_p.F:5-48, extrap_p_block.F:5-77
 *   p_ref_subtract / subtract_p    code/p_ref_subtract.F:6-100
 *   uvw_adv / uvw_adv_block        code/uvw_adv.F:5-63, uvw_adv_block.F:5-109
 *   swap_rhos_block                code/swap_rhos_block.F:5-51
 *   search_lib_block               code/search_lib_block.F:5-65
 *   slipbc / slipbc_block          code/slipbc.F:3-196
 * MPI_ALLREDUCE sums become block-order sums (one rank owns every block).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc_internal.h"

/* ---------------------------------------------------------------- coeff_p */
static void coeff_p_block(int nip1, int njp1, int nkp1, long jo, long ko,
                          const double *diu, const double *djv,
                          const double *rdiv, const double *rdju,
                          const double *didjp, const double *rp,
                          const double *dkp, const double *dkw, double *ap,
                          double *aw, double *ae, double *as, double *an,
                          double *al, double *ar, const int *bc)
{
    int ni = nip1 - 1, nj = njp1 - 1, nk = nkp1 - 1;
#define G(a, i, j) A2(a, i, j, nip1)
    /* starting surfaces (coeff_p_block.F:147-178) */
    for (int k = 2; k <= nk; k++)
        for (int j = 2; j <= nj; j++) A(ae, jo * (j - 1) + ko * (k - 1) + 1) = 0.;
    for (int k = 2; k <= nk; k++)
        for (int i = 2; i <= ni; i++) A(an, i + ko * (k - 1)) = 0.;
    for (int j = 2; j <= nj; j++)
        for (int i = 2; i <= ni; i++) A(ar, i + jo * (j - 1)) = 0.;
    /* coeff_p_block.F:182-215 */
    for (int j = 2; j <= nj; j++)
        for (int i = 2; i <= ni; i++) {
            double cef = G(rdju, i + 1, j) / G(diu, i + 1, j);
            double cnf = G(rdiv, i, j + 1) / G(djv, i, j + 1);
            double crf = G(didjp, i, j) / G(rp, i, j);
            long ijoff = i + jo * (j - 1) - ko;
            for (int k = 2; k <= nk; k++) {
                long ijk = ijoff + ko * k;
                A(aw, ijk) = A(ae, ijk - 1);
                A(ae, ijk) = cef * A(dkp, k);
                A(as, ijk) = A(an, ijk - jo);
                A(an, ijk) = cnf * A(dkp, k);
                A(al, ijk) = A(ar, ijk - ko);
                A(ar, ijk) = crf / A(dkw, k + 1);
                A(ap, ijk) = A(aw, ijk) + A(ae, ijk) + A(as, ijk) + A(an, ijk) +
                             A(al, ijk) + A(ar, ijk);
            }
        }
    /* faces (coeff_p_block.F:221-306) */
    if (bc[0] == ORC_BCT_PERIODIC || bc[0] == ORC_BCT_INTERFACE)
        for (int k = 2; k <= nk; k++)
            for (int j = 2; j <= nj; j++) {
                long ijk = jo * (j - 1) + ko * (k - 1) + 2;
                A(aw, ijk) = G(rdju, 2, j) / G(diu, 2, j) * A(dkp, k);
                A(ap, ijk) = A(ap, ijk) + A(aw, ijk);
            }
    if (bc[1] != ORC_BCT_PERIODIC && bc[1] != ORC_BCT_INTERFACE)
        for (int k = 2; k <= nk; k++)
            for (int j = 2; j <= nj; j++) {
                long ijk = jo * (j - 1) + ko * (k - 1) + ni;
                A(ap, ijk) = A(ap, ijk) - A(ae, ijk);
                A(ae, ijk) = 0.;
            }
    if (bc[2] == ORC_BCT_PERIODIC || bc[2] == ORC_BCT_INTERFACE)
        for (int k = 2; k <= nk; k++)
            for (int i = 2; i <= ni; i++) {
                long ijk = i + ko * (k - 1) + jo;
                A(as, ijk) = G(rdiv, i, 2) / G(djv, i, 2) * A(dkp, k);
                A(ap, ijk) = A(ap, ijk) + A(as, ijk);
            }
    if (bc[3] != ORC_BCT_PERIODIC && bc[3] != ORC_BCT_INTERFACE)
        for (int k = 2; k <= nk; k++)
            for (int i = 2; i <= ni; i++) {
                long ijk = i + ko * (k - 1) + jo * (nj - 1);
                A(ap, ijk) = A(ap, ijk) - A(an, ijk);
                A(an, ijk) = 0.;
            }
    if (bc[4] == ORC_BCT_PERIODIC || bc[4] == ORC_BCT_INTERFACE)
        for (int j = 2; j <= nj; j++)
            for (int i = 2; i <= ni; i++) {
                long ijk = i + jo * (j - 1) + ko;
                A(al, ijk) = G(didjp, i, j) / (G(rp, i, j) * A(dkw, 2));
                A(ap, ijk) = A(ap, ijk) + A(al, ijk);
            }
    if (bc[5] != ORC_BCT_PERIODIC && bc[5] != ORC_BCT_INTERFACE)
        for (int j = 2; j <= nj; j++)
            for (int i = 2; i <= ni; i++) {
                long ijk = i + jo * (j - 1) + ko * (nk - 1);
                A(ap, ijk) = A(ap, ijk) - A(ar, ijk);
                A(ar, ijk) = 0.;
            }
#undef G
}

void orc_coeff_p(orc_ctx *c, const double *diu, const double *djv,
                 const double *rdiv, const double *rdju, const double *didjp,
                 const double *rp, const double *dkp, const double *dkw,
                 double *ap, double *aw, double *ae, double *as, double *an,
                 double *al, double *ar)
{
    for (int lev = 1; lev <= c->nummgl; lev++)
        for (int b = 1; b <= c->numbl; b++) {
            int *n = c->mg_nijkp1[lev][b];
            long p1 = c->off1k[lev][b], p2 = c->off2[lev][b], p3 = c->off3[lev][b];
            coeff_p_block(n[0], n[1], n[2], n[0], (long)n[0] * n[1], diu + p2,
                          djv + p2, rdiv + p2, rdju + p2, didjp + p2, rp + p2,
                          dkp + p1, dkw + p1, ap + p3, aw + p3, ae + p3,
                          as + p3, an + p3, al + p3, ar + p3, c->bl_bc[b]);
        }
}

/* ----------------------------------------------------------------- sour_p */
static void sour_p_block(int nip1, int njp1, int nkp1, long jo, long ko,
                         double dtime, const double *diu, const double *djv,
                         const double *rdiv, const double *rdju,
                         const double *didjp, const double *dkp,
                         const double *u, const double *v, const double *w,
                         const double *rho, const double *rhonp1,
                         double *drhodt, double *s, double *srhot,
                         double *srhoux, double *gia, double *gja,
                         const double *rdidjp, const double *dkw)
{
    (void)diu;
    (void)djv;
    int ni = nip1 - 1, nj = njp1 - 1, nk = nkp1 - 1;
    double ddtime = 2.0 / (3.0 * dtime) * 0.5;
    double cdtime = 2.0 / (3.0 * dtime);
    double rdtime = 1.0 / dtime;
#define G(a, i, j) A2(a, i, j, nip1)
#define GJA(k, i) gja[((long)(k) - 1) + (long)nkp1 * ((long)(i) - 1)]
    for (int i = 2; i <= ni; i++) {
        double cnf = G(rdiv, i, 2);
        long ijoff = i + jo;
        for (int k = 2; k <= nk; k++) {
            long ijk = ijoff + ko * (k - 1);
            GJA(k, i) = cnf * A(dkp, k) * (A(rhonp1, ijk) + A(rhonp1, ijk - jo)) * A(v, ijk);
        }
    }
    for (int j = 2; j <= nj; j++) {
        long joff = jo * (j - 1);
        double cef = G(rdju, 2, j);
        for (int k = 2; k <= nk; k++) {
            long ijk = 2 + joff + ko * (k - 1);
            A(gia, k) = cef * A(dkp, k) * (A(rhonp1, ijk) + A(rhonp1, ijk - 1)) * A(u, ijk);
        }
        for (int i = 2; i <= ni; i++) {
            cef = G(rdju, i + 1, j);
            double cnf = G(rdiv, i, j + 1);
            double crf = G(didjp, i, j);
            long ijk = i + joff + ko;
            double grf = crf * (A(rhonp1, ijk) + A(rhonp1, ijk - ko)) * A(w, ijk);
            long ijoff = i + joff;
            for (int k = 2; k <= nk; k++) {
                ijk = ijoff + ko * (k - 1);
                long ijke = ijk + 1, ijkn = ijk + jo, ijkr = ijk + ko;
                double gwf = A(gia, k);
                double gef = cef * A(dkp, k) * (A(rhonp1, ijk) + A(rhonp1, ijke)) * A(u, ijke);
                A(gia, k) = gef;
                double gsf = GJA(k, i);
                double gnf = cnf * A(dkp, k) * (A(rhonp1, ijk) + A(rhonp1, ijkn)) * A(v, ijkn);
                GJA(k, i) = gnf;
                double glf = grf;
                grf = crf * (A(rhonp1, ijk) + A(rhonp1, ijkr)) * A(w, ijkr);
                A(s, ijk) = -ddtime * (gef - gwf + gnf - gsf + grf - glf);
                A(srhoux, ijk) = -ddtime * (gef - gwf + gnf - gsf + grf - glf);
                double vol = G(rdidjp, i, j) * A(dkw, k);
                A(drhodt, ijk) = (A(rhonp1, ijk) - A(rho, ijk)) * rdtime;
                A(s, ijk) = A(s, ijk) - cdtime * A(drhodt, ijk) * vol;
                A(srhot, ijk) = -cdtime * A(drhodt, ijk) * vol;
            }
        }
    }
#undef G
#undef GJA
}

void orc_sour_p(orc_ctx *c, double dtime, const double *diu,
                const double *djv, const double *rdiv, const double *rdju,
                const double *didjp, const double *dkp, const double *rdidjp,
                const double *dkw, const double *u, const double *v,
                const double *w, const double *rho, const double *rhonp1,
                double *drhodt, double *s, double *srhot, double *srhoux)
{
    int maxk = 0, maxik = 0;
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        if (n[2] > maxk) maxk = n[2];
        if (n[2] * n[0] > maxik) maxik = n[2] * n[0];
    }
    double *gia = (double *)calloc((size_t)maxk + 1, sizeof(double));
    double *gja = (double *)calloc((size_t)maxik + 1, sizeof(double));
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        long p1 = c->off1k[1][b], p2 = c->off2[1][b], p3 = c->off3[1][b];
        sour_p_block(n[0], n[1], n[2], n[0], (long)n[0] * n[1], dtime, diu + p2,
                     djv + p2, rdiv + p2, rdju + p2, didjp + p2, dkp + p1,
                     u + p3, v + p3, w + p3, rho + p3, rhonp1 + p3,
                     drhodt + p3, s + p3, srhot + p3, srhoux + p3, gia, gja,
                     rdidjp + p2, dkw + p1);
    }
    free(gia);
    free(gja);
}

/* ------------------------------------------------------------------ norms */
static void norms_block(const double *ap, const double *aw, const double *ae,
                        const double *as, const double *an, const double *al,
                        const double *ar, const double *x, const double *b,
                        double *residu, int nip1, int njp1, int nkp1,
                        const int *se, double *out)
{
    double rn = 0., fn = 0., en = 0., vn = 0.;
    long io = 1, jo = nip1, ko = (long)nip1 * njp1;
    (void)nkp1;
    for (int k = se[4]; k <= se[5]; k++) {
        long koff = ko * (k - 1);
        for (int j = se[2]; j <= se[3]; j++) {
            long jkoff = jo * (j - 1) + koff;
            for (int i = se[0]; i <= se[1]; i++) {
                long ijk = i + jkoff;
                double rhs = A(b, ijk);
                double var = A(x, ijk);
                double res = A(b, ijk) - A(ap, ijk) * var +
                             A(aw, ijk) * A(x, ijk - io) + A(ae, ijk) * A(x, ijk + io) +
                             A(as, ijk) * A(x, ijk - jo) + A(an, ijk) * A(x, ijk + jo) +
                             A(al, ijk) * A(x, ijk - ko) + A(ar, ijk) * A(x, ijk + ko);
                double err = res / A(ap, ijk);
                rn = rn + res * res;
                fn = fn + rhs * rhs;
                en = en + err * err;
                vn = vn + var * var;
                A(residu, ijk) = res;
            }
        }
    }
    out[0] = rn;
    out[1] = fn;
    out[2] = en;
    out[3] = vn;
}

void orc_norms(orc_ctx *c, int ilev, int mg_or_sg, const double *ap,
               const double *aw, const double *ae, const double *as,
               const double *an, const double *al, const double *ar,
               const double *x, const double *b, double *residu, double *out4)
{
    double r = 0., f = 0., e = 0., v = 0.;
    for (int bl = 1; bl <= c->numbl; bl++) {
        long p3 = c->off3[ilev][bl];
        long p3x = (mg_or_sg == 1) ? p3 : c->off3[1][bl];
        int *n = c->mg_nijkp1[ilev][bl];
        double o[4];
        norms_block(ap + p3, aw + p3, ae + p3, as + p3, an + p3, al + p3, ar + p3,
                    x + p3x, b + p3, residu + p3, n[0], n[1], n[2],
                    c->nijkse[ilev][bl], o);
        r = r + o[0];
        f = f + o[1];
        e = e + o[2];
        v = v + o[3];
    }
    double rn = 1. / c->npts_all[ilev];
    out4[0] = sqrt(r * rn);
    out4[1] = sqrt(f * rn);
    out4[2] = sqrt(e * rn);
    out4[3] = sqrt(v * rn);
    if (out4[3] == 0.) out4[3] = 1.;
}

/* ----------------------------------------------------------------- sporlx */
/* code/sporlx.F:211-275.  (io, jo, ko) and the coefficient order arrive
 * permuted for the j- and k-innermost passes, as sporlx passes them. */
static void spor(long io, long jo, long ko, int is, int ie, int js, int je,
                 int ks, int ke, double *f, const double *src,
                 const double *ap, const double *aw, const double *ae,
                 const double *as, const double *an, const double *al,
                 const double *ar, double omega, double *out)
{
    double resnrm = 0., errnrm = 0., varnrm = 0.;
    for (int k = ks; k <= ke; k++) {
        long koff = 1 + ko * (k - 1);
        for (int j = js; j <= je; j++) {
            long jkoff = jo * (j - 1) + koff;
            for (int i = is; i <= ie; i++) {
                long ijk = io * (i - 1) + jkoff;
                double f_old = A(f, ijk);
                double dx = (A(src, ijk) + A(aw, ijk) * A(f, ijk - io) +
                             A(ae, ijk) * A(f, ijk + io) + A(as, ijk) * A(f, ijk - jo) +
                             A(an, ijk) * A(f, ijk + jo) + A(al, ijk) * A(f, ijk - ko) +
                             A(ar, ijk) * A(f, ijk + ko)) /
                                A(ap, ijk) -
                            f_old;
                A(f, ijk) = f_old + omega * dx;
                dx = A(f, ijk) - f_old;
                double res = dx * A(ap, ijk);
                resnrm = resnrm + res * res;
                errnrm = errnrm + dx * dx;
                varnrm = varnrm + A(f, ijk) * A(f, ijk);
            }
        }
    }
    out[0] = resnrm;
    out[1] = errnrm;
    out[2] = varnrm;
}

/* code/sporlx.F:5-203 with niter = 1.  in/out4 = res, rhs, err, var norms. */
void orc_sporlx(orc_ctx *c, int ilev, const double *ap, const double *aw,
                const double *ae, const double *as, const double *an,
                const double *al, const double *ar, double *f,
                const double *b, double omega, double soltol, double *io4)
{
    double res_norm = io4[0], err_norm = io4[2], var_norm = io4[3];
    double rnpts_all = 1. / c->npts_all[ilev];
    int jumfor = ((c->jumble % 16) >= 8) ? 1 : 2;
    int jumst = (c->jumble % 24) / 8 + 1;
    int d[3];
    d[0] = jumst;
    d[1] = ORC_CYC(((jumfor + 1) % 2) + 1, jumst);
    d[2] = ORC_CYC((jumfor % 2) + 1, jumst);
    int isweep = 0;
    while (isweep < 1 && err_norm / var_norm > soltol) {
        isweep++;
        for (int il = 0; il < 3; il++) {
            int d1 = d[il];
            res_norm = 0.;
            err_norm = 0.;
            var_norm = 0.;
            for (int bl = 1; bl <= c->numbl; bl++) {
                int *n = c->mg_nijkp1[ilev][bl];
                long io = 1, jo = n[0], ko = (long)n[0] * n[1];
                int *se = c->nijkse[ilev][bl];
                long p3 = c->off3[ilev][bl];
                double o[3];
                if (d1 == 1)
                    spor(io, jo, ko, se[0], se[1], se[2], se[3], se[4], se[5], f + p3, b + p3,
                         ap + p3, aw + p3, ae + p3, as + p3, an + p3, al + p3, ar + p3, omega, o);
                else if (d1 == 2)
                    spor(jo, io, ko, se[2], se[3], se[0], se[1], se[4], se[5], f + p3, b + p3,
                         ap + p3, as + p3, an + p3, aw + p3, ae + p3, al + p3, ar + p3, omega, o);
                else
                    spor(ko, io, jo, se[4], se[5], se[0], se[1], se[2], se[3], f + p3, b + p3,
                         ap + p3, al + p3, ar + p3, aw + p3, ae + p3, as + p3, an + p3, omega, o);
                res_norm = res_norm + o[0];
                err_norm = err_norm + o[1];
                var_norm = var_norm + o[2];
            }
            orc_swap_sc(c, ilev, f, 1);
        }
        err_norm = sqrt(err_norm * rnpts_all);
        var_norm = sqrt(var_norm * rnpts_all);
        if (var_norm == 0.) var_norm = 1.;
    }
    res_norm = sqrt(res_norm * rnpts_all);
    c->jumble = c->jumble + 13;
    if (c->jumble > 99999) c->jumble = c->jumble % 99999;
    io4[0] = res_norm;
    io4[2] = err_norm;
    io4[3] = var_norm;
}

/* code/smooth.F:5-105, meth_smooth = 1 */
static void smooth(orc_ctx *c, int ilev, const double *ap, const double *aw,
                   const double *ae, const double *as, const double *an,
                   const double *al, const double *ar, double *f,
                   const double *b, double *residu, int nsmooth, double omega,
                   double soltol, double *nrm)
{
    if (ilev == 1 || ilev == c->nummgl) {
        orc_norms(c, ilev, 1, ap, aw, ae, as, an, al, ar, f, b, residu, nrm);
    } else {
        nrm[2] = 1.;
        nrm[3] = 1.;
    }
    int ismooth = 0;
    while (nrm[2] / nrm[3] > soltol && ismooth < nsmooth) {
        ismooth++;
        orc_sporlx(c, ilev, ap, aw, ae, as, an, al, ar, f, b, omega, soltol, nrm);
        if (ismooth == nsmooth)
            orc_norms(c, ilev, 1, ap, aw, ae, as, an, al, ar, f, b, residu, nrm);
    }
}

/* ------------------------------------------------------- grid transfers */
static void rest_block(const double *ff, double *fc, int nip1c, int njp1c,
                       int nkp1c, long joc, long koc, long jof, long kof,
                       int imult, int jmult, int kmult)
{
    double fac = 1.0;
    long iinc, jinc, kinc;
    if (imult == 1) { iinc = 0; fac = 0.5 * fac; } else iinc = -1;
    if (jmult == 1) { jinc = 0; fac = 0.5 * fac; } else jinc = -jof;
    if (kmult == 1) { kinc = 0; fac = 0.5 * fac; } else kinc = -kof;
    long offm11 = iinc, off1m1 = jinc, offmm1 = iinc + jinc, off11m = kinc;
    long offm1m = iinc + kinc, off1mm = jinc + kinc, offmmm = iinc + jinc + kinc;
    for (int k = 2; k <= nkp1c - 1; k++) {
        long koffc = koc * (k - 1), kofff = kof * (kmult * k - 2);
        for (int j = 2; j <= njp1c - 1; j++) {
            long jkoffc = joc * (j - 1) + koffc;
            long jkofff = jof * (jmult * j - 2) + kofff;
            for (int i = 2; i <= nip1c - 1; i++) {
                long ijkc = i + jkoffc;
                long ijkf = imult * i - 1 + jkofff;
                A(fc, ijkc) = fac * (A(ff, ijkf) + A(ff, ijkf + offm11) +
                                     A(ff, ijkf + off1m1) + A(ff, ijkf + offmm1) +
                                     A(ff, ijkf + off11m) + A(ff, ijkf + offm1m) +
                                     A(ff, ijkf + off1mm) + A(ff, ijkf + offmmm));
            }
        }
    }
}

void orc_restriction(orc_ctx *c, int ilev, const double *f, double *f1)
{
    int gc = ilev, gf = ilev - 1;
    for (int b = 1; b <= c->numbl; b++) {
        int *nc = c->mg_nijkp1[gc][b], *nf = c->mg_nijkp1[gf][b];
        int *m = c->mult[gf][b];
        rest_block(f + c->off3[gf][b], f1 + c->off3[gc][b], nc[0], nc[1], nc[2],
                   nc[0], (long)nc[0] * nc[1], nf[0], (long)nf[0] * nf[1], m[0],
                   m[1], m[2]);
    }
}

static const double c0 = 0.015625, c1i = 0.421875, c2i = 0.140625, c3i = 0.046875;

static void prol_block(double *ff, double *fc, double *cr, int nip1c,
                       int njp1c, int nkp1c, int nip1f, int njp1f, int nkp1f,
                       int imult, int jmult, int kmult, const int *bc)
{
    long joc = nip1c, koc = (long)nip1c * njp1c;
    long ijkoc[4] = {0, 1, joc, koc};
    int nijkp1c[4] = {0, nip1c, njp1c, nkp1c};
    long jof = nip1f, kof = (long)nip1f * njp1f;
    long eoffc = 1, noffc = joc, roffc = koc, neoffc = 1 + joc, nroffc = joc + koc;
    long eroffc = 1 + koc, enroffc = 1 + joc + koc;
    long eofff = 1, nofff = jof, rofff = kof, neofff = 1 + jof, nrofff = jof + kof;
    long erofff = 1 + kof, enrofff = 1 + jof + kof;
    /* coarse ghosts := interior neighbour on non-interface faces
     * (prol_block.F:325-357) */
    for (int is = 1; is <= 6; is++) {
        int d1 = (is + 1) / 2, d2 = ORC_CYC1(1, d1), d3 = ORC_CYC1(2, d1);
        int njt = nijkp1c[d2], nkt = nijkp1c[d3];
        long iot = ijkoc[d1], jot = ijkoc[d2], kot = ijkoc[d3];
        if (bc[is - 1] == ORC_BCT_INTERFACE) continue;
        long ioffc, inext;
        if (is % 2 == 1) { ioffc = 1; inext = iot; }
        else { ioffc = 1 + iot * (nijkp1c[d1] - 1); inext = -iot; }
        for (int kc = 1; kc <= nkt; kc++) {
            long koffc = ioffc + kot * (kc - 1);
            for (int jc = 1; jc <= njt; jc++) {
                long ijkc = jot * (jc - 1) + koffc;
                A(fc, ijkc) = A(fc, ijkc + inext);
            }
        }
    }
    for (long q = 1; q <= (long)nip1f * njp1f * nkp1f; q++) A(cr, q) = 0.;
    for (int kc = 1; kc <= nkp1c - 1; kc++) {
        int kf = kmult * kc - 1;
        long koffc = koc * (kc - 1), kofff = kof * (kf - 1);
        for (int jc = 1; jc <= njp1c - 1; jc++) {
            int jf = jmult * jc - 1;
            long jkoffc = joc * (jc - 1) + koffc, jkofff = jof * (jf - 1) + kofff;
            for (int ic = 1; ic <= nip1c - 1; ic++) {
                int if_ = imult * ic - 1;
                long ijkc = ic + jkoffc, ijkf = if_ + jkofff;
                double F0 = A(fc, ijkc), FE = A(fc, ijkc + eoffc), FN = A(fc, ijkc + noffc);
                double FR = A(fc, ijkc + roffc), FNE = A(fc, ijkc + neoffc);
                double FNR = A(fc, ijkc + nroffc), FER = A(fc, ijkc + eroffc);
                double FENR = A(fc, ijkc + enroffc);
                A(cr, ijkf) = A(cr, ijkf) + c1i * F0 + c2i * FE + c2i * FN + c2i * FR +
                              c3i * FNE + c3i * FNR + c3i * FER + c0 * FENR;
                A(cr, ijkf + eofff) = A(cr, ijkf + eofff) + c2i * F0 + c1i * FE + c3i * FN +
                                      c3i * FR + c2i * FNE + c0 * FNR + c2i * FER + c3i * FENR;
                A(cr, ijkf + nofff) = A(cr, ijkf + nofff) + c2i * F0 + c3i * FE + c1i * FN +
                                      c3i * FR + c2i * FNE + c2i * FNR + c0 * FER + c3i * FENR;
                A(cr, ijkf + rofff) = A(cr, ijkf + rofff) + c2i * F0 + c3i * FE + c3i * FN +
                                      c1i * FR + c0 * FNE + c2i * FNR + c2i * FER + c3i * FENR;
                A(cr, ijkf + neofff) = A(cr, ijkf + neofff) + c3i * F0 + c2i * FE + c2i * FN +
                                       c0 * FR + c1i * FNE + c3i * FNR + c3i * FER + c2i * FENR;
                A(cr, ijkf + nrofff) = A(cr, ijkf + nrofff) + c3i * F0 + c0 * FE + c2i * FN +
                                       c2i * FR + c3i * FNE + c1i * FNR + c3i * FER + c2i * FENR;
                A(cr, ijkf + erofff) = A(cr, ijkf + erofff) + c3i * F0 + c2i * FE + c0 * FN +
                                       c2i * FR + c3i * FNE + c3i * FNR + c1i * FER + c2i * FENR;
                A(cr, ijkf + enrofff) = A(cr, ijkf + enrofff) + c0 * F0 + c3i * FE + c3i * FN +
                                        c3i * FR + c2i * FNE + c2i * FNR + c2i * FER + c1i * FENR;
            }
        }
    }
    int is_ = (bc[0] == ORC_BCT_INTERFACE) ? 1 : 2;
    int ie = (bc[1] == ORC_BCT_INTERFACE) ? nip1f : nip1f - 1;
    int js = (bc[2] == ORC_BCT_INTERFACE) ? 1 : 2;
    int je = (bc[3] == ORC_BCT_INTERFACE) ? njp1f : njp1f - 1;
    int ks = (bc[4] == ORC_BCT_INTERFACE) ? 1 : 2;
    int ke = (bc[5] == ORC_BCT_INTERFACE) ? nkp1f : nkp1f - 1;
    for (int kf = ks; kf <= ke; kf++) {
        long kofff = kof * (kf - 1);
        for (int jf = js; jf <= je; jf++) {
            long jkofff = jof * (jf - 1) + kofff;
            for (int if_ = is_; if_ <= ie; if_++) {
                long ijkf = if_ + jkofff;
                A(ff, ijkf) = A(ff, ijkf) + A(cr, ijkf);
            }
        }
    }
}

void orc_prolongation(orc_ctx *c, int ilev, double *f)
{
    int gf = ilev, gc = ilev + 1;
    long maxn = 0;
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[gf][b];
        long t = (long)n[0] * n[1] * n[2];
        if (t > maxn) maxn = t;
    }
    double *cr = (double *)malloc(sizeof(double) * (size_t)(maxn + 1));
    for (int b = 1; b <= c->numbl; b++) {
        int *nc = c->mg_nijkp1[gc][b], *nf = c->mg_nijkp1[gf][b];
        int *m = c->mult[gf][b];
        prol_block(f + c->off3[gf][b], f + c->off3[gc][b], cr, nc[0], nc[1], nc[2],
                   nf[0], nf[1], nf[2], m[0], m[1], m[2], c->bl_bc[b]);
    }
    free(cr);
    orc_swap_sc(c, gf, f, 1);
}

static void init_level(orc_ctx *c, double *f, double value, int lev)
{
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[lev][b];
        long np = (long)n[0] * n[1] * n[2];
        for (long q = 0; q < np; q++) f[c->off3[lev][b] + q] = value;
    }
}

/* -------------------------------------------------------------- lmg_solve */
/* code/lmg_solve.F:5-172.  norms_out = rnorm, fnorm, enorm, vnorm of level
 * 1 followed by the number of finest-level visits (V-cycles). */
void orc_lmg_solve(orc_ctx *c, const orc_mgctrl *m, const double *ap,
                   const double *aw, const double *ae, const double *as,
                   const double *an, const double *al, const double *ar,
                   double *f, double *b, double *residu,
                   double *norms_out)
{
    int mg_gamma = (m->meth_cycle == 1) ? 1 : 2;
    int fcycle = (m->meth_cycle == 2);
    int nummgl = c->nummgl;
    double tolc = 0.;
    if (nummgl == 1) tolc = m->tolf;
    c->tolc = tolc;
    int nummg_l[ORC_MAXMGL + 2];
    double nrm[ORC_MAXMGL + 2][4];
    memset(nrm, 0, sizeof(nrm));
    orc_norms(c, 1, 1, ap, aw, ae, as, an, al, ar, f, b, residu, nrm[1]);
    nummg_l[1] = m->nummgits;
    int ilev = 1;
    int cycles = 0;
    while (nummg_l[1] > 0 && nrm[1][2] / nrm[1][3] > m->tolf) {
        int goto_fine = (ilev == nummgl) || (nummg_l[ilev] == 0);
        if (goto_fine) {
            if (ilev == nummgl) {
                /* solversc: the smoother as coarse solver (solversc.F:350-353) */
                smooth(c, ilev, ap, aw, ae, as, an, al, ar, f, b, residu, m->numcits,
                       m->relax_pmgc, tolc, nrm[ilev]);
                if (fcycle) mg_gamma = 1;
            }
            if (ilev > 1 && nummgl != 1) {
                ilev = ilev - 1;
                orc_prolongation(c, ilev, f);
                smooth(c, ilev, ap, aw, ae, as, an, al, ar, f, b, residu, m->numpost,
                       m->relax_pmg, tolc, nrm[ilev]);
                if (ilev == 1 && fcycle) mg_gamma = 2;
            }
            if (ilev == 1) cycles++;
            nummg_l[ilev] = nummg_l[ilev] - 1;
        } else {
            smooth(c, ilev, ap, aw, ae, as, an, al, ar, f, b, residu, m->numpre,
                   m->relax_pmg, tolc, nrm[ilev]);
            ilev = ilev + 1;
            nummg_l[ilev] = mg_gamma;
            init_level(c, f, 0., ilev);
            orc_restriction(c, ilev, residu, b);
        }
    }
    for (int lev = 1; lev <= nummgl; lev++) {
        c->rnorm[lev] = nrm[lev][0];
        c->fnorm[lev] = nrm[lev][1];
        c->enorm[lev] = nrm[lev][2];
        c->vnorm[lev] = nrm[lev][3];
    }
    for (int q = 0; q < 4; q++) norms_out[q] = nrm[1][q];
    norms_out[4] = cycles;
}

/* ------------------------------------------------------- post-processing */
void orc_extrap_p(orc_ctx *c, double *p)
{
    /* co = cyclic1 (extrap_p_block.F:317) */
    static const int co[2][4] = {{0, 2, 1, 1}, {0, 3, 3, 2}};
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        double *pb = p + c->off3[1][b];
        long ijko[4] = {0, 1, n[0], (long)n[0] * n[1]};
        int ijkbc[7] = {0, 1, n[0], 1, n[1], 1, n[2]};
        int nijk[4] = {0, n[0], n[1], n[2]};
        for (int s = 1; s <= 6; s++) {
            int t = c->bl_bc[b][s - 1];
            if (t == ORC_BCT_INTERFACE || t == ORC_BCT_PERIODIC) continue;
            int d1 = (s + 1) / 2, d2 = co[0][d1], d3 = co[1][d1];
            long io = ijko[d1], io1 = (s % 2 == 0) ? -io : io;
            long jo = ijko[d2], ko = ijko[d3];
            int i = ijkbc[s];
            long ioff = 1 + io * (i - 1);
            for (int k = 1; k <= nijk[d3]; k++) {
                long koff = ioff + ko * (k - 1);
                for (int j = 1; j <= nijk[d2]; j++) {
                    long ijk = jo * (j - 1) + koff;
                    A(pb, ijk) = A(pb, ijk + io1);
                }
            }
        }
    }
    orc_swap_sc(c, 1, p, 1);
}

void orc_p_ref_subtract(orc_ctx *c, double *p)
{
    int *n = c->mg_nijkp1[1][1];
    double p_ref = A(p, c->off3[1][1] + 2 + n[0] * (2 - 1) + (long)n[0] * n[1] * (2 - 1));
    for (int b = 1; b <= c->numbl; b++) {
        int *nb = c->mg_nijkp1[1][b];
        double *pb = p + c->off3[1][b];
        long np = (long)nb[0] * nb[1] * nb[2];
        for (long q = 0; q < np; q++) pb[q] = pb[q] - p_ref;
    }
}

void orc_uvw_adv(orc_ctx *c, int ivar, double dtime, const double *diu,
                 const double *rp, const double *dkw, double *u,
                 const double *u_int, const double *rho, const double *p)
{
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        int nip1 = n[0], njp1 = n[1], nkp1 = n[2];
        int *bcb = c->bl_bc[b];
        /* set_loop_bound(ivar1, 1, 1, iblk, iblk, 1, ijkse) */
        int istr = (ivar == ORC_SV_U && bcb[0] != ORC_BCT_PERIODIC && bcb[0] != ORC_BCT_INTERFACE) ? 3 : 2;
        int jstr = (ivar == ORC_SV_V && bcb[2] != ORC_BCT_PERIODIC && bcb[2] != ORC_BCT_INTERFACE) ? 3 : 2;
        int kstr = (ivar == ORC_SV_W && bcb[4] != ORC_BCT_PERIODIC && bcb[4] != ORC_BCT_INTERFACE) ? 3 : 2;
        long p3 = c->off3[1][b], p2 = c->off2[1][b], p1 = c->off1k[1][b];
        double *ub = u + p3;
        const double *uib = u_int + p3, *rb = rho + p3, *pb = p + p3;
        const double *dg = diu + p2, *rpb = rp + p2, *dkwb = dkw + p1;
        int ni = nip1 - 1, nj = njp1 - 1, nk = nkp1 - 1;
        long jo = nip1, ko = (long)nip1 * njp1;
        double ddtime = 1.5 * dtime;
        if (ivar != ORC_SV_W) {
            long iojo = (ivar == ORC_SV_U) ? 1 : jo;
            for (int k = kstr; k <= nk; k++) {
                long koff = ko * (k - 1);
                for (int j = jstr; j <= nj; j++) {
                    long jkoff = jo * (j - 1) + koff, joff_ij = (long)nip1 * (j - 1);
                    for (int i = istr; i <= ni; i++) {
                        long ijk = i + jkoff, ijkw = ijk - iojo, ij = i + joff_ij;
                        double dpdi = (A(pb, ijk) - A(pb, ijkw)) / A(dg, ij);
                        double rhou = 0.5 * (A(rb, ijk) + A(rb, ijkw));
                        A(ub, ijk) = A(uib, ijk) - ddtime * dpdi / rhou;
                    }
                }
            }
        } else {
            for (int k = kstr; k <= nk; k++) {
                long koff = ko * (k - 1);
                for (int j = jstr; j <= nj; j++) {
                    long jkoff = jo * (j - 1) + koff, joff_ij = (long)nip1 * (j - 1);
                    for (int i = jstr; i <= ni; i++) {
                        long ijk = i + jkoff, ijkl = ijk - ko, ij = i + joff_ij;
                        double dpdi = (A(pb, ijk) - A(pb, ijkl)) / (A(rpb, ij) * A(dkwb, k));
                        double rhou = 0.5 * (A(rb, ijk) + A(rb, ijkl));
                        A(ub, ijk) = A(uib, ijk) - ddtime * dpdi / rhou;
                    }
                }
            }
        }
    }
    orc_swap_sc(c, 1, u, 2);
}

void orc_swap_rhos(orc_ctx *c, double *rho, double *rhonp1, double *rhonm1)
{
    for (long q = 0; q < c->tot_sg3; q++) {
        rhonm1[q] = rho[q];
        rho[q] = rhonp1[q];
    }
}

/* code/search_lib.F:277-338 + search_lib_block.F:5-65 (Temperature is not
 * written by the block routine and is left out here) */
void orc_search_lib(orc_ctx *c, double *sc1, double *rhonp1, double alpha,
                    const double *rho, double rholo, double rhohi)
{
    for (long q = 0; q < c->tot_sg3; q++) {
        double rho_mix = 1.0 / (sc1[q] / rhohi + (1.0 - sc1[q]) / rholo);
        if (sc1[q] > 1.0) rho_mix = rhohi;
        if (sc1[q] < 0.0) rho_mix = rholo;
        double rho_tmp = rho_mix;
        rhonp1[q] = alpha * rho[q] + (1.0 - alpha) * rho_tmp;
        sc1[q] = (sc1[q] * rho[q]) / rhonp1[q];
        if (sc1[q] > 1.0) sc1[q] = 1.0;
    }
    orc_swap_sc(c, 1, sc1, 2);
    orc_swap_sc(c, 1, rhonp1, 2);
}

/* code/slipbc.F:59-190 (TRACTION and ZERO_GRAD faces on j sides) */
void orc_slipbc(orc_ctx *c, double dtime, const double *djp, double *u,
                double *v, const double *v_int, double *w, double *sc1,
                double *rho, const double *p)
{
    double ddtime = 1.5 * dtime;
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        int nip1 = n[0], njp1 = n[1], nkp1 = n[2];
        long jo = nip1, ko = (long)nip1 * njp1, p3 = c->off3[1][b], p2 = c->off2[1][b];
        double *ub = u + p3, *vb = v + p3, *wb = w + p3, *sb = sc1 + p3, *rb = rho + p3;
        const double *vib = v_int + p3, *pb = p + p3, *dj = djp + p2;
        int *bcb = c->bl_bc[b];
        if (bcb[2] == ORC_BCT_TRACTION)
            for (int i = 1; i <= nip1; i++)
                for (int k = 2; k <= nkp1 - 1; k++) {
                    long ijk = i + jo * (2 - 1) + ko * (k - 1), ijks = ijk - jo;
                    A(sb, ijks) = A(sb, ijk);
                    A(rb, ijks) = A(rb, ijk);
                    double rhou = 0.5 * (A(rb, ijk) + A(rb, ijks));
                    A(ub, ijks) = A(ub, ijk);
                    A(vb, ijk) = A(vib, ijk) - ddtime * ((2.0 * A(pb, ijk) - 2.0 * 0.0) / A2(dj, i, 1, nip1)) / rhou;
                    A(vb, ijks) = A(vb, ijk);
                    A(wb, ijks) = A(wb, ijk);
                }
        if (bcb[3] == ORC_BCT_TRACTION)
            for (int i = 1; i <= nip1; i++)
                for (int k = 2; k <= nkp1 - 1; k++) {
                    long ijk = i + jo * (njp1 - 2) + ko * (k - 1), ijkn = ijk + jo;
                    A(sb, ijkn) = A(sb, ijk);
                    A(rb, ijkn) = A(rb, ijk);
                    double rhou = 0.5 * (A(rb, ijk) + A(rb, ijkn));
                    A(ub, ijkn) = A(ub, ijk);
                    A(vb, ijkn) = A(vib, ijkn) - ddtime * ((-2.0 * A(pb, ijk) + 2.0 * 0.0) / A2(dj, i, njp1 - 1, nip1)) / rhou;
                    A(wb, ijkn) = A(wb, ijk);
                }
        if (bcb[2] == ORC_BCT_ZERO_GRAD)
            for (int i = 1; i <= nip1; i++)
                for (int k = 2; k <= nkp1 - 1; k++) {
                    long ijk = i + jo * (2 - 1) + ko * (k - 1), ijks = ijk - jo;
                    A(sb, ijks) = A(sb, ijk);
                    A(rb, ijks) = A(rb, ijk);
                    A(ub, ijks) = A(ub, ijk);
                    A(vb, ijk) = 0.0;
                    A(vb, ijks) = A(vb, ijk);
                    A(wb, ijks) = A(wb, ijk);
                }
        if (bcb[3] == ORC_BCT_ZERO_GRAD)
            for (int i = 1; i <= nip1; i++)
                for (int k = 2; k <= nkp1 - 1; k++) {
                    long ijk = i + jo * (njp1 - 2) + ko * (k - 1), ijkn = ijk + jo;
                    A(sb, ijkn) = A(sb, ijk);
                    A(rb, ijkn) = A(rb, ijk);
                    A(ub, ijkn) = A(ub, ijk);
                    A(vb, ijkn) = 0.0;
                    A(wb, ijkn) = A(wb, ijk);
                }
    }
}
