/*
 * orc_virtbc.c -- oracle: wall ghost velocities (log law) and the van
 * Driest damping field.  TEST INFRASTRUCTURE ONLY.
 *
 *   set_virt_bc        code/set_virt_bc.F:8-276
 *   set_virt_bc_block  code/set_virt_bc_block.F:12-456 (velocity branches)
 * Every call first resets vd_damping to 1 on every point of every block
 * (set_virt_bc.F:73-75); init_vdd is set for all sides by the u call.
 * One deviation: the u south/north branch averages rho over i-1 and i, and
 * at i = 1 the reference reads the element before the slice (outside the
 * block at the very first point); here rho(i) is used there instead.  That
 * only touches the corner ghost (1, 1, 1) and the damping of ghost column
 * i = 1, which nothing reads.
 */
#include <math.h>
#include "orc_internal.h"

enum { M_DIP, M_DIU, M_DIV, M_DIX, M_RDIP, M_RDIV, M_RDIX, M_DJP, M_DJU, M_DJV, M_DJX, M_RDJP,
       M_RDJU, M_RDJX, M_HIJP, M_HJIP, M_HKIP, M_HKJP, M_HIJU, M_HJIU, M_HKIU, M_HKJU, M_HIJV,
       M_HJIV, M_HKIV, M_HKJV, M_RP, M_RU, M_RV, M_DIDJP, M_RDIDJP, M_DIDJU, M_RDIDJU, M_DJDIV,
       M_RDJDIV };

typedef struct {
    double visc, kappa, aplus, ylaminar, value;
} vbc_par;

static double fsign1(double b) { return b >= 0.0 ? 1.0 : -1.0; } /* SIGN(1., b) */

/* init_vdd[block][side] lives with the context of the caller (the u call
 * sets it); kept here per oracle library instance */
static int g_init_vdd[ORC_MAXBL + 1][6];

/* one side of one block: code/set_virt_bc_block.F, velocity branches */
static void vbc_side(int iva, int side, const int *n, long off3, double *f, const double *rho,
                     double *vdd, const double *tw, double *const *M, const double *dkp,
                     const double *dkw, int *init_vdd, const vbc_par *P)
{
    long ijko[4] = {0, 1, n[0], (long)n[0] * n[1]};
    int nijk[4] = {0, n[0], n[1], n[2]};
    int d3 = (side + 1) / 2, d1 = ORC_CYC1(1, d3), d2 = ORC_CYC1(2, d3);
    long io = ijko[d1], jo = ijko[d2], ko = ijko[d3];
    int nip1 = nijk[d1], njp1 = nijk[d2], nkp1 = nijk[d3];
    int k, k1;
    long kko;
    if (side % 2 == 1) { k = 1; k1 = 2; kko = ko; }
    else { k = nkp1; k1 = nkp1; kko = -ko; }
    int wallef = side == 2, wallnf = side == 4, wallrf = side == 6;
    double wewall = wallef ? -1. : 1., snwall = wallnf ? -1. : 1., lrwall = wallrf ? -1. : 1.;
    long koff = 1 + ko * (k - 1);
    double *F = f + off3, *V = vdd + off3;
    const double *R = rho + off3;
    double visc = P->visc, kappa = P->kappa, aplus = P->aplus, ylam = P->ylaminar, value = P->value;
#define M2(a, q) A(M[a], q)
    if (iva == ORC_SV_U && (side == 3 || side == 4)) {
        int kstart, kfinish, kstep, kstr;
        if (k1 == 2) { kstart = k1; kfinish = k1 + nkp1 / 2; kstep = 1; kstr = k1 + 1; }
        else { kstart = k1; kfinish = k1 - nkp1 / 2; kstep = -1; kstr = k1 - 1; }
        long koff0 = (long)nip1 * (k1 - 1);
        if (init_vdd[side - 1]) {
            init_vdd[side - 1] = 0;
            for (int kvd = kstart; kstep > 0 ? kvd <= kfinish : kvd >= kfinish; kvd += kstep) {
                int kref = (k1 == 2) ? kvd - 1 : kvd;
                long koff2 = 1 + ko * (kref - 1);
                for (int j = 1; j <= njp1; j++)
                    for (int i = 1; i <= nip1; i++) A(V, io * (i - 1) + jo * (j - 1) + koff2 + kko) = 0.;
            }
        }
        for (int kvd = kstart; kstep > 0 ? kvd <= kfinish : kvd >= kfinish; kvd += kstep) {
            int kref = (k1 == 2) ? kvd - 1 : kvd;
            long koff2 = 1 + ko * (kref - 1);
            for (int j = 1; j <= njp1; j++) {
                long jkoff = jo * (j - 1) + koff2;
                for (int i = 1; i <= nip1; i++) {
                    long ijk = io * (i - 1) + jkoff, nx = ijk + kko;
                    double rw = (i > 1) ? A(R, ijk - io) : A(R, ijk);
                    double rwn = (i > 1) ? A(R, nx - io) : A(R, nx);
                    double rhof = 0.25 * (A(R, ijk) + A(R, nx) + rw + rwn);
                    double twv = A(tw, j + (long)njp1 * (i - 1));
                    double tw_mean = fabs(twv);
                    double ut = sqrt(tw_mean / rhof);
                    double dist = 0.5 * M2(M_DJU, i + koff0);
                    if (kvd != kstart)
                        for (int kk = kstr; kstep > 0 ? kk <= kvd : kk >= kvd; kk += kstep)
                            dist = dist + M2(M_DJX, i + (long)nip1 * (kk - 1));
                    double yp = dist * ut * rhof / visc;
                    double d = 1. - exp(-yp / aplus);
                    A(V, nx) = d < 1.0 ? d : 1.0;
                    if (kvd == kstart) {
                        if (yp > ylam)
                            A(F, ijk) = A(F, nx) - snwall * fsign1(twv) * ut * M2(M_DJX, i + koff0) / (kappa * dist);
                        else
                            A(F, ijk) = 2. * value - A(F, nx);
                    }
                }
            }
        }
        return;
    }
    if (init_vdd[side - 1]) {
        init_vdd[side - 1] = 0;
        for (int j = 1; j <= njp1; j++) {
            long jkoff = jo * (j - 1) + koff + kko;
            for (int i = 1; i <= nip1; i++) A(V, io * (i - 1) + jkoff) = 0.;
        }
    }
    /* loop order: j outer / i inner for (u, L/R) and (v, W/E); i outer /
     * j inner with rhoflast reset per i for (v, L/R), (w, W/E), (w, S/N) */
    int i_outer = (iva == ORC_SV_V && side >= 5) || iva == ORC_SV_W;
    for (int a = 1; a <= (i_outer ? nip1 : njp1); a++) {
        double rl = A(R, koff + (i_outer ? 0 : jo * (a - 1)));
        double rln = A(R, koff + (i_outer ? 0 : jo * (a - 1)) + kko);
        for (int bq = 1; bq <= (i_outer ? njp1 : nip1); bq++) {
            int i = i_outer ? a : bq, j = i_outer ? bq : a;
            long ijk = io * (i - 1) + jo * (j - 1) + koff, nx = ijk + kko;
            double rhof = 0.25 * (A(R, ijk) + A(R, nx) + rl + rln);
            rl = A(R, ijk);
            rln = A(R, nx);
            /* f = f_next - wsgn*sign(1,tw)*ut*m1*m2/(kappa*dist), evaluated
             * left to right as in the source (m2 = 1 where absent) */
            double dist, twv, wsgn, m1, m2 = 1.0;
            if (iva == ORC_SV_U) { /* L/R */
                long ij = i + (long)nip1 * (j - 1);
                dist = 0.5 * M2(M_RU, ij) * A(dkp, k1);
                twv = A(tw, ij);
                wsgn = lrwall;
                m1 = M2(M_RU, ij);
                m2 = A(dkw, k1);
            } else if (iva == ORC_SV_V && side <= 2) {
                long q = k1 + (long)nkp1 * (i - 1);
                dist = 0.5 * M2(M_DIV, q);
                twv = A(tw, j + (long)njp1 * (i - 1));
                wsgn = wewall;
                m1 = M2(M_DIX, q);
            } else if (iva == ORC_SV_V) { /* L/R */
                long ij = i + (long)nip1 * (j - 1);
                dist = 0.5 * M2(M_RV, ij) * A(dkp, k1);
                twv = A(tw, ij);
                wsgn = lrwall;
                m1 = M2(M_RV, ij);
                m2 = A(dkw, k1);
            } else if (side <= 2) { /* w, W/E */
                long q = k1 + (long)nkp1 * (i - 1);
                dist = 0.5 * M2(M_DIP, q);
                twv = A(tw, j + (long)njp1 * (i - 1));
                wsgn = wewall;
                m1 = M2(M_DIU, q);
            } else { /* w, S/N */
                long q = i + (long)nip1 * (k1 - 1);
                dist = 0.5 * M2(M_DJP, q);
                twv = A(tw, j + (long)njp1 * (i - 1));
                wsgn = snwall;
                m1 = M2(M_DJV, q);
            }
            double tw_mean = fabs(twv);
            double ut = sqrt(tw_mean / rhof);
            double yp = dist * ut * rhof / visc;
            double d = 1. - exp(-yp / aplus);
            A(V, nx) = d > A(V, nx) ? d : A(V, nx);
            if (yp > ylam)
                A(F, ijk) = A(F, nx) - wsgn * fsign1(twv) * ut * m1 * m2 / (kappa * dist);
            else
                A(F, ijk) = 2. * value - A(F, nx);
        }
    }
#undef M2
}

/* code/set_virt_bc.F:55-273 at level 1.  tw[0..3] are the wall arrays the
 * step passes for this component: u -> tw_sfi, tw_nfi, tw_lfi, tw_rfi;
 * v -> tw_wfj, tw_efj, tw_lfj, tw_rfj; w -> tw_wfk, tw_efk, tw_sfk, tw_nfk. */
void orc_set_virt_bc(orc_ctx *c, int iva, double visc, double kappa, double aplus,
                     double ylaminar, double *f, const double *rho, double *vdd,
                     const double *metric, const double *dkp, const double *dkw,
                     double *const *tw)
{
    vbc_par P = {visc, kappa, aplus, ylaminar, 0.0};
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        long p3 = c->off3[1][b], p2 = c->off2[1][b], p1 = c->off1k[1][b];
        if (iva == ORC_SV_U)
            for (int s = 0; s < 6; s++) g_init_vdd[b][s] = 1;
        for (long q = 0; q < (long)n[0] * n[1] * n[2]; q++) vdd[p3 + q] = 1.0;
        double *M[ORC_NMETRIC];
        for (int q = 0; q < ORC_NMETRIC; q++) M[q] = (double *)metric + (long)q * c->tot2 + p2;
        for (int s = 1; s <= 6; s++) {
            int t = c->bl_bc[b][s - 1];
            int d3 = (s + 1) / 2;
            if (t == ORC_BCT_INTERFACE || t == ORC_BCT_PERIODIC || iva == d3) continue;
            if (t != ORC_BCT_WALL) continue; /* velocities: only wall sides call the block */
            const double *twp;
            if (iva == ORC_SV_U)
                twp = (s == 3) ? tw[0] + c->offki[1][b] : (s == 4) ? tw[1] + c->offki[1][b]
                      : (s == 5) ? tw[2] + p2 : tw[3] + p2;
            else if (iva == ORC_SV_V)
                twp = (s == 1) ? tw[0] + c->offjk[1][b] : (s == 2) ? tw[1] + c->offjk[1][b]
                      : (s == 5) ? tw[2] + p2 : tw[3] + p2;
            else
                twp = (s == 1) ? tw[0] + c->offjk[1][b] : (s == 2) ? tw[1] + c->offjk[1][b]
                      : (s == 3) ? tw[2] + c->offki[1][b] : tw[3] + c->offki[1][b];
            vbc_side(iva, s, n, p3, f, rho, vdd, twp, M, dkp + p1, dkw + p1, g_init_vdd[b], &P);
        }
    }
}
