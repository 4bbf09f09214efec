/*
 * orc_metric.c -- oracle: staggered-grid metrics.  TEST INFRASTRUCTURE ONLY.
 *
 * Restates comp_metric (code/comp_metric.F:5-255) for one rank:
 * metric_block (code/metric_block2.F:9-280) for every block of a level,
 * then metric_swap1 / metric_swap2 (code/metric_swap1.F, metric_swap2.F)
 * -- pack every periodic/interface face, then unpack.
 */
#include <math.h>
#include <stdlib.h>
#include "orc_internal.h"

enum { M_DIP, M_DIU, M_DIV, M_DIX, M_RDIP, M_RDIV, M_RDIX, M_DJP, M_DJU,
       M_DJV, M_DJX, M_RDJP, M_RDJU, M_RDJX, M_HIJP, M_HJIP, M_HKIP, M_HKJP,
       M_HIJU, M_HJIU, M_HKIU, M_HKJU, M_HIJV, M_HJIV, M_HKIV, M_HKJV, M_RP,
       M_RU, M_RV, M_DIDJP, M_RDIDJP, M_DIDJU, M_RDIDJU, M_DJDIV, M_RDJDIV };

/* the 34 arrays moved by metric_swap1/2 (rdidjp is not among them) */
static const int swapped[34] = {
    M_DIP, M_DIU, M_DIV, M_DIX, M_RDIP, M_RDIV, M_RDIX, M_DJP, M_DJU, M_DJV,
    M_DJX, M_RDJP, M_RDJU, M_RDJX, M_HIJP, M_HJIP, M_HKIP, M_HKJP, M_HIJU,
    M_HJIU, M_HKIU, M_HKJU, M_HIJV, M_HJIV, M_HKIV, M_HKJV, M_RP, M_RU, M_RV,
    M_DIDJP, M_DIDJU, M_RDIDJU, M_DJDIV, M_RDJDIV};

/* code/metric_block2.F:9-280.  m[k] points at metric array k of this block. */
static void metric_block(int nip1, int njp1, int nkp1, const double *x,
                         const double *y, const double *t, double **m,
                         double *dkp, double *dkw, int gotrad)
{
    const int nip2 = nip1 + 1;
    const double tiny = 1.0e-30;
    for (int k = 0; k < ORC_NMETRIC; k++)
        for (long q = 0; q < (long)nip1 * njp1; q++) m[k][q] = 0.;
    for (int k = 1; k <= nkp1; k++) { A(dkp, k) = 0.; A(dkw, k) = 0.; }
    double rad_on = gotrad ? 1. : 0.;
    double rad_off = 1. - rad_on;
    double y_ij = 0, y_ijp1 = 0, y_ip1j = 0;
#define X(i, j) A2(x, i, j, nip2)
#define Y(i, j) A2(y, i, j, nip2)
#define M(a, i, j) A2(m[a], i, j, nip1)
    for (int j = 1; j <= njp1; j++)
        for (int i = 1; i <= nip1; i++) {
            int ip1 = i + 1 < nip1 ? i + 1 : nip1;
            int im1 = i - 1 > 1 ? i - 1 : 1;
            int jp1 = j + 1 < njp1 ? j + 1 : njp1;
            int jm1 = j - 1 > 1 ? j - 1 : 1;
            double x_ij = X(i, j), x_ip1j = X(ip1, j), x_ijp1 = X(i, jp1);
            double x_ip1jp1 = X(ip1, jp1), x_im1j = X(im1, j);
            double x_im1jp1 = X(im1, jp1), x_ijm1 = X(i, jm1);
            double x_ip1jm1 = X(ip1, jm1);
            y_ij = Y(i, j);
            y_ip1j = Y(ip1, j);
            y_ijp1 = Y(i, jp1);
            double y_ip1jp1 = Y(ip1, jp1), y_im1j = Y(im1, j);
            double y_im1jp1 = Y(im1, jp1), y_ijm1 = Y(i, jm1);
            double y_ip1jm1 = Y(ip1, jm1);

            double xu_ij = 0.5 * (x_ij + x_ijp1), yu_ij = 0.5 * (y_ij + y_ijp1);
            double xu_ijm1 = 0.5 * (x_ij + x_ijm1), yu_ijm1 = 0.5 * (y_ij + y_ijm1);
            double xu_ip1j = 0.5 * (x_ip1j + x_ip1jp1), yu_ip1j = 0.5 * (y_ip1j + y_ip1jp1);
            double xv_ij = 0.5 * (x_ij + x_ip1j), yv_ij = 0.5 * (y_ij + y_ip1j);
            double xv_im1j = 0.5 * (x_ij + x_im1j), yv_im1j = 0.5 * (y_ij + y_im1j);
            double xv_ijp1 = 0.5 * (x_ijp1 + x_ip1jp1), yv_ijp1 = 0.5 * (y_ijp1 + y_ip1jp1);
            double xp_ij = 0.25 * (x_ij + x_ip1j + x_ijp1 + x_ip1jp1);
            double yp_ij = 0.25 * (y_ij + y_ip1j + y_ijp1 + y_ip1jp1);
            double xp_ijm1 = 0.25 * (x_ij + x_ip1j + x_ijm1 + x_ip1jm1);
            double yp_ijm1 = 0.25 * (y_ij + y_ip1j + y_ijm1 + y_ip1jm1);
            double xp_im1j = 0.25 * (x_ij + x_im1j + x_ijp1 + x_im1jp1);
            double yp_im1j = 0.25 * (y_ij + y_im1j + y_ijp1 + y_im1jp1);

            double rp_ij = yp_ij * rad_on + rad_off;
            double ru_ij = yu_ij * rad_on + rad_off;
            double rv_ij = yv_ij * rad_on + rad_off;
            double rx_ij = y_ij * rad_on + rad_off;
            M(M_RU, i, j) = ru_ij;
            M(M_RV, i, j) = rv_ij;
            M(M_RP, i, j) = rp_ij;

            M(M_DIP, i, j) = sqrt((xu_ip1j - xu_ij) * (xu_ip1j - xu_ij) +
                                  (yu_ip1j - yu_ij) * (yu_ip1j - yu_ij));
            M(M_DIU, i, j) = sqrt((xp_ij - xp_im1j) * (xp_ij - xp_im1j) +
                                  (yp_ij - yp_im1j) * (yp_ij - yp_im1j));
            M(M_DIV, i, j) = sqrt((x_ip1j - x_ij) * (x_ip1j - x_ij) +
                                  (y_ip1j - y_ij) * (y_ip1j - y_ij));
            M(M_DIX, i, j) = sqrt((xv_ij - xv_im1j) * (xv_ij - xv_im1j) +
                                  (yv_ij - yv_im1j) * (yv_ij - yv_im1j));
            M(M_RDIP, i, j) = rp_ij * M(M_DIP, i, j);
            M(M_RDIV, i, j) = rv_ij * M(M_DIV, i, j);
            M(M_RDIX, i, j) = rx_ij * M(M_DIX, i, j);

            M(M_DJP, i, j) = sqrt((xv_ijp1 - xv_ij) * (xv_ijp1 - xv_ij) +
                                  (yv_ijp1 - yv_ij) * (yv_ijp1 - yv_ij));
            M(M_DJU, i, j) = sqrt((x_ijp1 - x_ij) * (x_ijp1 - x_ij) +
                                  (y_ijp1 - y_ij) * (y_ijp1 - y_ij));
            M(M_DJV, i, j) = sqrt((xp_ij - xp_ijm1) * (xp_ij - xp_ijm1) +
                                  (yp_ij - yp_ijm1) * (yp_ij - yp_ijm1));
            M(M_DJX, i, j) = sqrt((xu_ij - xu_ijm1) * (xu_ij - xu_ijm1) +
                                  (yu_ij - yu_ijm1) * (yu_ij - yu_ijm1));
            M(M_RDJP, i, j) = rp_ij * M(M_DJP, i, j);
            M(M_RDJU, i, j) = ru_ij * M(M_DJU, i, j);
            M(M_RDJX, i, j) = rx_ij * M(M_DJX, i, j);

            M(M_DIDJP, i, j) = M(M_DIP, i, j) * M(M_DJP, i, j);
            M(M_DIDJU, i, j) = M(M_DIU, i, j) * M(M_DJU, i, j);
            M(M_DJDIV, i, j) = M(M_DJV, i, j) * M(M_DIV, i, j);
            M(M_RDIDJP, i, j) = rp_ij * M(M_DIDJP, i, j);
            M(M_RDIDJU, i, j) = M(M_DIU, i, j) * M(M_RDJU, i, j);
            M(M_RDJDIV, i, j) = M(M_DJV, i, j) * M(M_RDIV, i, j);
        }
    for (int k = 1; k <= nkp1; k++) {
        int kp1 = k + 1 < nkp1 ? k + 1 : nkp1;
        int km1 = k - 1 > 1 ? k - 1 : 1;
        A(dkp, k) = A(t, kp1) - A(t, k);
        A(dkw, k) = (A(t, kp1) - A(t, km1)) * 0.5;
    }
    /* y_ijp1, y_ij, y_ip1j keep their values from the last (nip1, njp1)
     * point of the loop above, exactly as in metric_block2.F:258-277 */
    for (int j = 2; j <= njp1 - 1; j++)
        for (int i = 2; i <= nip1 - 1; i++) {
            M(M_HIJP, i, j) = (M(M_DIV, i, j + 1) - M(M_DIV, i, j)) / (M(M_DIDJP, i, j) + tiny);
            M(M_HJIP, i, j) = (M(M_DJU, i + 1, j) - M(M_DJU, i, j)) / (M(M_DIDJP, i, j) + tiny);
            M(M_HKIP, i, j) = (M(M_RU, i + 1, j) - M(M_RU, i, j)) / (M(M_RDIP, i, j) + tiny);
            M(M_HKJP, i, j) = (M(M_RV, i, j + 1) - M(M_RV, i, j)) / (M(M_RDJP, i, j) + tiny);
            M(M_HIJU, i, j) = (M(M_DIX, i, j + 1) - M(M_DIX, i, j)) / (M(M_DIDJU, i, j) + tiny);
            M(M_HJIU, i, j) = (M(M_DJP, i, j) - M(M_DJP, i - 1, j)) / (M(M_DIDJU, i, j) + tiny);
            M(M_HKIU, i, j) = (M(M_RP, i, j) - M(M_RP, i - 1, j)) / (M(M_RU, i, j) * M(M_DIU, i, j) + tiny);
            M(M_HKJU, i, j) = (y_ijp1 - y_ij) * rad_on / (M(M_RDJU, i, j) + tiny);
            M(M_HIJV, i, j) = (M(M_DIP, i, j) - M(M_DIP, i, j - 1)) / (M(M_DJDIV, i, j) + tiny);
            M(M_HJIV, i, j) = (M(M_DJX, i + 1, j) - M(M_DJX, i, j)) / (M(M_DJDIV, i, j) + tiny);
            M(M_HKIV, i, j) = (y_ip1j - y_ij) * rad_on / (M(M_RDIV, i, j) + tiny);
            M(M_HKJV, i, j) = (M(M_RP, i, j) - M(M_RP, i, j - 1)) / (M(M_RV, i, j) * M(M_DJV, i, j) + tiny);
        }
#undef X
#undef Y
#undef M
}

/* metric_swap1: pack face `s` of a block into buf; returns values written */
static long metric_pack(int s, int bc, int nip1, int njp1, int nkp1, double **m,
                        const double *dkp, const double *dkw, double *buf)
{
    long p = 0;
    if (bc != ORC_BCT_INTERFACE && bc != ORC_BCT_PERIODIC) return 0;
    if (s == 5) { buf[p++] = A(dkp, 2); buf[p++] = A(dkw, 2); return p; }
    if (s == 6) { buf[p++] = A(dkp, nkp1 - 1); buf[p++] = A(dkw, nkp1 - 1); return p; }
    int i, je; long io, jo;
    if (s == 1) { i = 2; io = 1; jo = nip1; je = njp1; }
    else if (s == 2) { i = nip1 - 1; io = 1; jo = nip1; je = njp1; }
    else if (s == 3) { i = 2; io = nip1; jo = 1; je = nip1; }
    else { i = njp1 - 1; io = nip1; jo = 1; je = nip1; }
    long ioff = 1 + io * (i - 1);
    for (int j = 1; j <= je; j++) {
        long ij = ioff + jo * (j - 1);
        for (int q = 0; q < 34; q++) buf[p++] = A(m[swapped[q]], ij);
    }
    return p;
}

/* metric_swap2: unpack into the ghost line of face `s` */
static void metric_unpack(int s, int bc, int nip1, int njp1, int nkp1, double **m,
                          double *dkp, double *dkw, const double *buf)
{
    long p = 0;
    if (bc != ORC_BCT_INTERFACE && bc != ORC_BCT_PERIODIC) return;
    if (s == 5) { A(dkp, 1) = buf[p++]; A(dkw, 1) = buf[p++]; return; }
    if (s == 6) { A(dkp, nkp1) = buf[p++]; A(dkw, nkp1) = buf[p++]; return; }
    int i, je; long io, jo;
    if (s == 1) { i = 1; io = 1; jo = nip1; je = njp1; }
    else if (s == 2) { i = nip1; io = 1; jo = nip1; je = njp1; }
    else if (s == 3) { i = 1; io = nip1; jo = 1; je = nip1; }
    else { i = njp1; io = nip1; jo = 1; je = nip1; }
    long ioff = 1 + io * (i - 1);
    for (int j = 1; j <= je; j++) {
        long ij = ioff + jo * (j - 1);
        for (int q = 0; q < 34; q++) A(m[swapped[q]], ij) = buf[p++];
    }
}

void orc_comp_metric(orc_ctx *c, const double *x, const double *y,
                     const double *z, double *metric, double *dkp,
                     double *dkw, int gotrad)
{
    /* one pack buffer slot per (block, side) */
    long maxface = 0;
    for (int b = 1; b <= c->numbl; b++) {
        int *n = c->mg_nijkp1[1][b];
        long f = 34L * (n[0] > n[1] ? n[0] : n[1]) + 2;
        if (f > maxface) maxface = f;
    }
    double *slots = (double *)calloc((size_t)maxface * 6 * (c->numbl + 1), sizeof(double));
    for (int lev = 1; lev <= c->nummgl; lev++) {
        for (int b = 1; b <= c->numbl; b++) {
            int *n = c->mg_nijkp1[lev][b];
            double *m[ORC_NMETRIC];
            for (int k = 0; k < ORC_NMETRIC; k++) m[k] = metric + (long)k * c->tot2 + c->off2[lev][b];
            metric_block(n[0], n[1], n[2], x + c->offxy[lev][b], y + c->offxy[lev][b],
                         z + c->offz[lev][b], m, dkp + c->off1k[lev][b],
                         dkw + c->off1k[lev][b], gotrad);
        }
        /* pack: the slot of the partner face (comp_metric.F:113-118) */
        for (int b = 1; b <= c->numbl; b++) {
            int *n = c->mg_nijkp1[lev][b];
            double *m[ORC_NMETRIC];
            for (int k = 0; k < ORC_NMETRIC; k++) m[k] = metric + (long)k * c->tot2 + c->off2[lev][b];
            for (int s = 1; s <= 6; s++) {
                int bn = c->bl2bl[b][s - 1], sn = c->bl2side[b][s - 1];
                if (bn <= 0) continue;
                double *slot = slots + ((long)(bn * 6 + (sn - 1))) * maxface;
                metric_pack(s, c->bl_bc[b][s - 1], n[0], n[1], n[2], m,
                            dkp + c->off1k[lev][b], dkw + c->off1k[lev][b], slot);
            }
        }
        for (int b = 1; b <= c->numbl; b++) {
            int *n = c->mg_nijkp1[lev][b];
            double *m[ORC_NMETRIC];
            for (int k = 0; k < ORC_NMETRIC; k++) m[k] = metric + (long)k * c->tot2 + c->off2[lev][b];
            for (int s = 1; s <= 6; s++) {
                if (c->bl2bl[b][s - 1] <= 0) continue;
                const double *slot = slots + ((long)(b * 6 + (s - 1))) * maxface;
                metric_unpack(s, c->bl_bc[b][s - 1], n[0], n[1], n[2], m,
                              dkp + c->off1k[lev][b], dkw + c->off1k[lev][b], slot);
            }
        }
    }
    free(slots);
}
