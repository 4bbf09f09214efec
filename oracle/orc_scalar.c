/*
 * orc_scalar.c -- oracle: mixture-fraction transport and its boundary
 * values.  TEST INFRASTRUCTURE ONLY.
 *
 *   set_gamsc1_bc   code/set_gamsc1_bc.F (gamlam, ghost diffusivities, the
 *                   interface gradients of tvdgrad.inc)
 *   set_sc1         code/set_sc1.F:5-95, set_sc1_block.F:5-511: TVD
 *                   convection + diffusion, AB2, updating sc1 IN PLACE in
 *                   the loop order j, i, k, so later points read already
 *                   updated lower neighbours (kept exactly)
 *   set_sc1_bc      code/set_sc1_bc.F
 *   set_sc1var      code/set_sc1var.F, set_sc1var_block.F
 * The interface gradient arrays of tvdgrad.inc are sized here by the
 * blocks (the reference fixes them at 66 x 258 x 303).
 */
#include <math.h>
#include <stdlib.h>
#include "orc_internal.h"

enum { M_DIP, M_DIU, M_DIV, M_DIX, M_RDIP, M_RDIV, M_RDIX, M_DJP, M_DJU, M_DJV, M_DJX, M_RDJP,
       M_RDJU, M_RDJX, M_HIJP, M_HJIP, M_HKIP, M_HKJP, M_HIJU, M_HJIU, M_HKIU, M_HKJU, M_HIJV,
       M_HJIV, M_HKIV, M_HKJV, M_RP, M_RU, M_RV, M_DIDJP, M_RDIDJP, M_DIDJU, M_RDIDJU, M_DJDIV,
       M_RDJDIV };

/* per-block face gradients (tvdgrad.inc): dfdxw/dfdxe (j, k), dfdys/dfdyn
 * (i, k), dfdzl/dfdzr (i, j), each nijk-max squared */
typedef struct {
    long stride;  /* per block */
    int m;        /* leading dimension */
    double *xw, *xe, *ys, *yn, *zl, *zr;
} grads;

static grads g_grads;

static void grads_alloc(orc_ctx *c)
{
    int m = 0;
    for (int b = 1; b <= c->numbl; b++)
        for (int d = 0; d < 3; d++)
            if (c->mg_nijkp1[1][b][d] > m) m = c->mg_nijkp1[1][b][d];
    long need = (long)m * m * (c->numbl + 1);
    if (g_grads.m != m || g_grads.stride * (c->numbl + 1) < need) {
        free(g_grads.xw); free(g_grads.xe); free(g_grads.ys); free(g_grads.yn);
        free(g_grads.zl); free(g_grads.zr);
        g_grads.m = m;
        g_grads.stride = (long)m * m;
        g_grads.xw = calloc(need, sizeof(double));
        g_grads.xe = calloc(need, sizeof(double));
        g_grads.ys = calloc(need, sizeof(double));
        g_grads.yn = calloc(need, sizeof(double));
        g_grads.zl = calloc(need, sizeof(double));
        g_grads.zr = calloc(need, sizeof(double));
    }
}

#define GR(arr, b, x, y) (g_grads.arr[(long)(b) * g_grads.stride + ((long)(x) - 1) + (long)g_grads.m * ((long)(y) - 1)])

/* code/set_gamsc1_bc.F */
void orc_set_gamsc1_bc(orc_ctx *c, double visc, const double *sc1, double *gamsc1,
                       double *gamlam, const double *metric, const double *dkp)
{
    grads_alloc(c);
    const double sclam = 0.72;
    for (long q = 0; q < c->tot_sg3; q++) gamlam[q] = visc / sclam;
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        int nip1 = n[0], njp1 = n[1], nkp1 = n[2];
        int ni = nip1 - 1, nj = njp1 - 1, nk = nkp1 - 1;
        long jo = nip1, ko = (long)nip1 * njp1;
        double *s = (double *)sc1 + c->off3[1][b];
        double *g = gamsc1 + c->off3[1][b], *gl = gamlam + c->off3[1][b];
        const double *diu = metric + (long)M_DIU * c->tot2 + c->off2[1][b];
        const double *djv = metric + (long)M_DJV * c->tot2 + c->off2[1][b];
        const double *rp = metric + (long)M_RP * c->tot2 + c->off2[1][b];
        const double *dk = dkp + c->off1k[1][b];
        int *bc = c->bl_bc[b];
        for (int j = 2; j <= nj; j++)
            for (int k = 2; k <= nk; k++) {
                long jk = jo * (j - 1) + ko * (k - 1);
                long ij1 = 3 + jo * (j - 1);
                long ijkw = 1 + jk, ijk = 2 + jk, ijk1 = ijk + 1, ijk2 = ni + jk;
                GR(xw, b, j, k) = (A(s, ijk1) - A(s, ijk)) / A(diu, ij1);
                if (bc[0] == ORC_BCT_PERIODIC) A(g, ijkw) = A(g, ijk2);
                else if (bc[0] == ORC_BCT_WALL) { A(g, ijkw) = -A(g, ijk); A(gl, ijkw) = -A(gl, ijk); }
                else if (bc[0] != ORC_BCT_INTERFACE) A(g, ijkw) = A(g, ijk);
                ij1 = ni + jo * (j - 1);
                long ijke = nip1 + jk;
                ijk = ijke - 1;
                ijk1 = ijk - 1;
                ijk2 = 2 + jk;
                GR(xe, b, j, k) = (A(s, ijk) - A(s, ijk1)) / A(diu, ij1);
                if (bc[1] == ORC_BCT_PERIODIC) A(g, ijke) = A(g, ijk2);
                else if (bc[1] == ORC_BCT_WALL) { A(g, ijke) = -A(g, ijk); A(gl, ijke) = -A(gl, ijk); }
                else if (bc[1] != ORC_BCT_INTERFACE) A(g, ijke) = A(g, ijk);
            }
        for (int i = 2; i <= ni; i++)
            for (int k = 2; k <= nk; k++) {
                long ik = i + ko * (k - 1);
                long ij1 = i + jo * (3 - 1);
                long ijks = ik, ijk = ik + jo, ijk1 = ijk + jo, ijk2 = ik + jo * (nj - 1);
                GR(ys, b, i, k) = (A(s, ijk1) - A(s, ijk)) / A(djv, ij1);
                if (bc[2] == ORC_BCT_PERIODIC) A(g, ijks) = A(g, ijk2);
                else if (bc[2] == ORC_BCT_WALL) { A(g, ijks) = -A(g, ijk); A(gl, ijks) = -A(gl, ijk); }
                else if (bc[2] != ORC_BCT_INTERFACE) A(g, ijks) = A(g, ijk);
                ij1 = i + jo * (nj - 1);
                long ijkn = ik + jo * (njp1 - 1);
                ijk = ijkn - jo;
                ijk1 = ijk - jo;
                ijk2 = ik + jo;
                GR(yn, b, i, k) = (A(s, ijk) - A(s, ijk1)) / A(djv, ij1);
                if (bc[3] == ORC_BCT_PERIODIC) A(g, ijkn) = A(g, ijk2);
                else if (bc[3] == ORC_BCT_WALL) { A(g, ijkn) = -A(g, ijk); A(gl, ijkn) = -A(gl, ijk); }
                else if (bc[3] != ORC_BCT_INTERFACE) A(g, ijkn) = A(g, ijk);
            }
        for (int j = 2; j <= nj; j++)
            for (int i = 2; i <= ni; i++) {
                long ij = i + jo * (j - 1);
                long ij1 = i + jo * (j - 1);
                long ijkl = ij, ijk = ij + ko, ijk1 = ijk + ko, ijk2 = ij + ko * (nk - 1);
                GR(zl, b, i, j) = (A(s, ijk1) - A(s, ijk)) / (A(rp, ij1) * A(dk, 2));
                if (bc[4] == ORC_BCT_PERIODIC) A(g, ijkl) = A(g, ijk2);
                else if (bc[4] == ORC_BCT_WALL) { A(g, ijkl) = -A(g, ijk); A(gl, ijkl) = -A(gl, ijk); }
                else if (bc[4] != ORC_BCT_INTERFACE) A(g, ijkl) = A(g, ijk);
                long ijkr = ij + ko * (nkp1 - 1);
                ijk = ijkr - ko;
                ijk1 = ijk - ko;
                ijk2 = ij + ko;
                GR(zr, b, i, j) = (A(s, ijk) - A(s, ijk1)) / (A(rp, ij1) * A(dk, nk - 1));
                if (bc[5] == ORC_BCT_PERIODIC) A(g, ijkr) = A(g, ijk2);
                else if (bc[5] == ORC_BCT_WALL) { A(g, ijkr) = -A(g, ijk); A(gl, ijkr) = -A(gl, ijk); }
                else if (bc[5] != ORC_BCT_INTERFACE) A(g, ijkr) = A(g, ijk);
            }
    }
}

static inline double fmin_(double a, double b) { return a < b ? a : b; }
static inline double fmax_(double a, double b) { return a > b ? a : b; }

/* code/set_sc1_block.F:66-505 */
static void set_sc1_block(orc_ctx *c, int b, double dtime, double *const *M, const double *dkp,
                          const double *dkw, const double *u, const double *v, const double *w,
                          double *sc1, double *hsc1, const double *rho, const double *gamsc1,
                          const double *gamlam)
{
    const double lambda = 4.0, small = 1.e-30;
    int *n = c->mg_nijkp1[1][b];
    int nip1 = n[0], njp1 = n[1], nkp1 = n[2];
    int ni = nip1 - 1, nj = njp1 - 1, nk = nkp1 - 1;
    long io = 1, jo = nip1, ko = (long)nip1 * njp1;
    int *bc = c->bl_bc[b];
#define G(a, i, j) A2(M[a], i, j, nip1)
    for (int j = 2; j <= nj; j++)
        for (int i = 2; i <= ni; i++)
            for (int k = 2; k <= nk; k++) {
                long ijk = i + jo * (j - 1) + ko * (k - 1);
                long ijkw = ijk - io, ijke = ijk + io, ijks = ijk - jo, ijkn = ijk + jo;
                long ijkl = ijk - ko, ijkr = ijk + ko;
                double rhowf = 0.5 * (A(rho, ijk) + A(rho, ijkw));
                double rhoef = 0.5 * (A(rho, ijk) + A(rho, ijke));
                double rhosf = 0.5 * (A(rho, ijk) + A(rho, ijks));
                double rhonf = 0.5 * (A(rho, ijk) + A(rho, ijkn));
                double rholf = 0.5 * (A(rho, ijk) + A(rho, ijkl));
                double rhorf = 0.5 * (A(rho, ijk) + A(rho, ijkr));
                double rhop = A(rho, ijk);
                double gamwf = 0.5 * (A(gamsc1, ijk) + A(gamsc1, ijkw)) * rhowf + 0.5 * (A(gamlam, ijk) + A(gamlam, ijkw));
                double gamef = 0.5 * (A(gamsc1, ijk) + A(gamsc1, ijke)) * rhoef + 0.5 * (A(gamlam, ijk) + A(gamlam, ijke));
                double gamsf = 0.5 * (A(gamsc1, ijk) + A(gamsc1, ijks)) * rhosf + 0.5 * (A(gamlam, ijk) + A(gamlam, ijks));
                double gamnf = 0.5 * (A(gamsc1, ijk) + A(gamsc1, ijkn)) * rhonf + 0.5 * (A(gamlam, ijk) + A(gamlam, ijkn));
                double gamlf = 0.5 * (A(gamsc1, ijk) + A(gamsc1, ijkl)) * rholf + 0.5 * (A(gamlam, ijk) + A(gamlam, ijkl));
                double gamrf = 0.5 * (A(gamsc1, ijk) + A(gamsc1, ijkr)) * rhorf + 0.5 * (A(gamlam, ijk) + A(gamlam, ijkr));
                double uwf = A(u, ijk), uef = A(u, ijke), vsf = A(v, ijk), vnf = A(v, ijkn);
                double wlf = A(w, ijk), wrf = A(w, ijkr);
                double dfdxwf = (A(sc1, ijk) - A(sc1, ijkw)) / G(M_DIU, i, j);
                double dfdxef = (A(sc1, ijke) - A(sc1, ijk)) / G(M_DIU, i + 1, j);
                double dfdxwwf, dfdxeef, dfdyssf, dfdynnf, dfdzllf, dfdzrrf;
                if (i == 2) {
                    if (bc[0] != ORC_BCT_INTERFACE) dfdxwwf = dfdxwf;
                    else dfdxwwf = GR(xe, c->bl2bl[b][0], j, k);
                } else {
                    dfdxwwf = (A(sc1, ijkw) - A(sc1, ijkw - io)) / G(M_DIU, i - 1, j);
                }
                if (i == ni) {
                    if (bc[1] != ORC_BCT_INTERFACE) dfdxeef = dfdxef;
                    else dfdxeef = GR(xw, c->bl2bl[b][1], j, k);
                } else {
                    dfdxeef = (A(sc1, ijke + io) - A(sc1, ijke)) / G(M_DIU, i + 2, j);
                }
                double dfdysf = (A(sc1, ijk) - A(sc1, ijks)) / G(M_DJV, i, j);
                double dfdynf = (A(sc1, ijkn) - A(sc1, ijk)) / G(M_DJV, i, j + 1);
                if (j == 2) {
                    if (bc[2] != ORC_BCT_INTERFACE) dfdyssf = dfdysf;
                    else dfdyssf = GR(yn, c->bl2bl[b][2], i, k);
                } else {
                    dfdyssf = (A(sc1, ijks) - A(sc1, ijks - jo)) / G(M_DJV, i, j - 1);
                }
                if (j == nj) {
                    if (bc[3] != ORC_BCT_INTERFACE) dfdynnf = dfdynf;
                    else dfdynnf = GR(ys, c->bl2bl[b][3], i, k);
                } else {
                    dfdynnf = (A(sc1, ijkn + jo) - A(sc1, ijkn)) / G(M_DJV, i, j + 2);
                }
                double dfdzlf = (A(sc1, ijk) - A(sc1, ijkl)) / (G(M_RP, i, j) * A(dkp, k - 1));
                double dfdzrf = (A(sc1, ijkr) - A(sc1, ijk)) / (G(M_RP, i, j) * A(dkp, k));
                if (k == 2) {
                    if (bc[4] != ORC_BCT_INTERFACE) dfdzllf = dfdzlf;
                    else dfdzllf = GR(zr, c->bl2bl[b][4], i, j);
                } else {
                    dfdzllf = (A(sc1, ijkl) - A(sc1, ijkl - ko)) / (G(M_RP, i, j) * A(dkp, k - 2));
                }
                if (k == nk) {
                    if (bc[5] != ORC_BCT_INTERFACE) dfdzrrf = dfdzrf;
                    else dfdzrrf = GR(zl, c->bl2bl[b][5], i, j);
                } else {
                    dfdzrrf = (A(sc1, ijkr + ko) - A(sc1, ijkr)) / (G(M_RP, i, j) * A(dkp, k + 1));
                }
                double rwst = (uwf >= 0.0) ? (dfdxwwf + small) / (dfdxwf + small) : (dfdxef + small) / (dfdxwf + small);
                double rest = (uef > 0.0) ? (dfdxwf + small) / (dfdxef + small) : (dfdxeef + small) / (dfdxef + small);
                double rsth = (vsf >= 0.0) ? (dfdyssf + small) / (dfdysf + small) : (dfdynf + small) / (dfdysf + small);
                double rnth = (vnf > 0.0) ? (dfdysf + small) / (dfdynf + small) : (dfdynnf + small) / (dfdynf + small);
                double rlft = (wlf >= 0.0) ? (dfdzllf + small) / (dfdzlf + small) : (dfdzrf + small) / (dfdzlf + small);
                double rrht = (wrf > 0.0) ? (dfdzlf + small) / (dfdzrf + small) : (dfdzrrf + small) / (dfdzrf + small);
                double limw = fmax_(0.0, fmin_(lambda * rwst, 1.0));
                double lime = fmax_(0.0, fmin_(lambda * rest, 1.0));
                double lims = fmax_(0.0, fmin_(lambda * rsth, 1.0));
                double limn = fmax_(0.0, fmin_(lambda * rnth, 1.0));
                double liml = fmax_(0.0, fmin_(lambda * rlft, 1.0));
                double limr = fmax_(0.0, fmin_(lambda * rrht, 1.0));
                double s0 = A(sc1, ijk);
                double fwf, fef, fsf, fnf, flf, frf;
                if (uwf > 0.0) fwf = A(sc1, ijkw) + 0.5 * limw * (s0 - A(sc1, ijkw));
                else if (uwf < 0.0) fwf = s0 + 0.5 * limw * (A(sc1, ijkw) - s0);
                else fwf = 0.5 * (s0 + A(sc1, ijkw));
                if (uef > 0.0) fef = s0 + 0.5 * lime * (A(sc1, ijke) - s0);
                else if (uef < 0.0) fef = A(sc1, ijke) + 0.5 * lime * (s0 - A(sc1, ijke));
                else fef = 0.5 * (s0 + A(sc1, ijke));
                if (vsf > 0.0) fsf = A(sc1, ijks) + 0.5 * lims * (s0 - A(sc1, ijks));
                else if (vsf < 0.0) fsf = s0 + 0.5 * lims * (A(sc1, ijks) - s0);
                else fsf = 0.5 * (s0 + A(sc1, ijks));
                if (vnf > 0.0) fnf = s0 + 0.5 * limn * (A(sc1, ijkn) - s0);
                else if (vnf < 0.0) fnf = A(sc1, ijkn) + 0.5 * limn * (s0 - A(sc1, ijkn));
                else fnf = 0.5 * (s0 + A(sc1, ijkn));
                if (wlf > 0.0) flf = A(sc1, ijkl) + 0.5 * liml * (s0 - A(sc1, ijkl));
                else if (wlf < 0.0) flf = s0 + 0.5 * liml * (A(sc1, ijkl) - s0);
                else flf = 0.5 * (s0 + A(sc1, ijkl));
                if (wrf > 0.0) frf = s0 + 0.5 * limr * (A(sc1, ijkr) - s0);
                else if (wrf < 0.0) frf = A(sc1, ijkr) + 0.5 * limr * (s0 - A(sc1, ijkr));
                else frf = 0.5 * (s0 + A(sc1, ijkr));
                double areawf = G(M_RDJU, i, j) * A(dkw, k);
                double areaef = G(M_RDJU, i + 1, j) * A(dkw, k);
                double areasf = G(M_RDIV, i, j) * A(dkw, k);
                double areanf = G(M_RDIV, i, j + 1) * A(dkw, k);
                double areak = G(M_DIDJP, i, j);
                double vol = G(M_RDIDJP, i, j) * A(dkw, k);
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
                double sc1tmp = s0 + dtime / (vol * rhop) * (1.5 * h - 0.5 * A(hsc1, ijk));
                A(hsc1, ijk) = h;
                if (sc1tmp < 0.0) sc1tmp = 0.0;
                if (sc1tmp > 1.0) sc1tmp = 1.0;
                A(sc1, ijk) = sc1tmp;
            }
#undef G
}

void orc_set_sc1(orc_ctx *c, double dtime, const double *metric, const double *dkp,
                 const double *dkw, const double *u, const double *v, const double *w,
                 double *sc1, double *hsc1, const double *rho, const double *gamsc1,
                 const double *gamlam)
{
    for (int b = 1; b <= c->numbl; b++) {
        long p3 = c->off3[1][b], p2 = c->off2[1][b], p1 = c->off1k[1][b];
        double *M[ORC_NMETRIC];
        for (int q = 0; q < ORC_NMETRIC; q++) M[q] = (double *)metric + (long)q * c->tot2 + p2;
        set_sc1_block(c, b, dtime, M, dkp + p1, dkw + p1, u + p3, v + p3, w + p3, sc1 + p3,
                      hsc1 + p3, rho + p3, gamsc1 + p3, gamlam + p3);
    }
    orc_swap_sc(c, 1, sc1, 2);
}

/* code/set_sc1_bc.F */
void orc_set_sc1_bc(orc_ctx *c, double *f)
{
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        int nip1 = n[0], njp1 = n[1], nkp1 = n[2];
        int ni = nip1 - 1, nj = njp1 - 1, nk = nkp1 - 1;
        long jo = nip1, ko = (long)nip1 * njp1;
        double *s = f + c->off3[1][b];
        int *bc = c->bl_bc[b];
#define COPY(side, ghost, inner, per)                                                        \
    do {                                                                                     \
        if (bc[side] == ORC_BCT_PERIODIC) A(s, ghost) = A(s, per);                           \
        else if (bc[side] != ORC_BCT_INTERFACE && bc[side] != ORC_BCT_FIXED) A(s, ghost) = A(s, inner); \
    } while (0)
        for (int j = 2; j <= nj; j++)
            for (int k = 2; k <= nk; k++) {
                long jk = jo * (j - 1) + ko * (k - 1);
                COPY(0, 1 + jk, 2 + jk, ni + jk);
                COPY(1, nip1 + jk, nip1 - 1 + jk, 2 + jk);
            }
        for (int i = 2; i <= ni; i++)
            for (int k = 2; k <= nk; k++) {
                long ik = i + ko * (k - 1);
                COPY(2, ik, ik + jo, ik + jo * (nj - 1));
                COPY(3, ik + jo * (njp1 - 1), ik + jo * (njp1 - 2), ik + jo);
            }
        for (int j = 2; j <= nj; j++)
            for (int i = 2; i <= ni; i++) {
                long ij = i + jo * (j - 1);
                COPY(4, ij, ij + ko, ij + ko * (nk - 1));
                COPY(5, ij + ko * (nkp1 - 1), ij + ko * (nkp1 - 2), ij + ko);
            }
#undef COPY
    }
}

/* code/set_sc1var.F, set_sc1var_block.F:26-66 */
void orc_set_sc1var(orc_ctx *c, const double *sc1, double *sc1var, const double *metric,
                    const double *dkp, const double *dkw)
{
    const double cfv = 0.1;
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        int nip1 = n[0], njp1 = n[1], nkp1 = n[2];
        long jo = nip1, ko = (long)nip1 * njp1;
        const double *s = sc1 + c->off3[1][b];
        double *sv = sc1var + c->off3[1][b];
        const double *dip = metric + (long)M_DIP * c->tot2 + c->off2[1][b];
        const double *djp = metric + (long)M_DJP * c->tot2 + c->off2[1][b];
        const double *rp = metric + (long)M_RP * c->tot2 + c->off2[1][b];
        const double *dk = dkp + c->off1k[1][b], *dw = dkw + c->off1k[1][b];
        for (int k = 2; k <= nkp1 - 1; k++)
            for (int j = 2; j <= njp1 - 1; j++)
                for (int i = 2; i <= nip1 - 1; i++) {
                    long ijk = i + jo * (j - 1) + ko * (k - 1);
                    double fwf = 0.5 * (A(s, ijk) + A(s, ijk - 1));
                    double fef = 0.5 * (A(s, ijk) + A(s, ijk + 1));
                    double fsf = 0.5 * (A(s, ijk) + A(s, ijk - jo));
                    double fnf = 0.5 * (A(s, ijk) + A(s, ijk + jo));
                    double flf = 0.5 * (A(s, ijk) + A(s, ijk - ko));
                    double frf = 0.5 * (A(s, ijk) + A(s, ijk + ko));
                    double dfdip = (fef - fwf) / A2(dip, i, j, nip1);
                    double dfdjp = (fnf - fsf) / A2(djp, i, j, nip1);
                    double dfdkp = (frf - flf) / (A2(rp, i, j, nip1) * A(dw, k));
                    double dfdijk = dfdip * dfdip + dfdjp * dfdjp + dfdkp * dfdkp;
                    double di = A2(dip, i, j, nip1), dj = A2(djp, i, j, nip1);
                    double dk_ = A2(rp, i, j, nip1) * A(dk, k);
                    double delta = pow(di * dj * dk_, .33333333);
                    A(sv, ijk) = cfv * dfdijk * (delta * delta);
                }
    }
    orc_swap_sc(c, 1, sc1var, 2);
}
