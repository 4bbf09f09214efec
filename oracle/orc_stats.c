/*
 * orc_stats.c -- oracle: span-averaged running statistics.
 * TEST INFRASTRUCTURE ONLY.
 *
 *   statistics  code/statistics.F:1-200 (the averaging part; the z-line and
 *               file outputs are not restated)
 *   centre      code/statistics.F:335-467
 *   dim_ave     code/field_out.F (dim = 3: the mean over k = 2..nkp1-1)
 *
 * Outputs are per block 2-D (i, j) arrays in the level-1 2-D metric layout.
 * statistics.F indexes them with an offset (ioffxy) it never sets; here each
 * block's own (i, j) offset is used.  centre leaves the edge cells of its
 * cell-centred copies unset (the reference's work arrays keep whatever they
 * held); here they are 0.
 */
#include <stdlib.h>
#include "orc_internal.h"

/* code/statistics.F:335-467 on one block: cell-centred velocities */
static void centre(int nip1, int njp1, int nkp1, const double *u, const double *v, const double *w, double *ut,
                   double *vt, double *wt)
{
    int ni = nip1 - 1, nj = njp1 - 1, nk = nkp1 - 1;
    long jo = nip1, ko = (long)nip1 * njp1;
    for (int k = 2; k <= nk; k++)
        for (int j = 2; j <= nj; j++)
            for (int i = 2; i <= ni; i++) {
                long ijk = i + jo * (j - 1) + ko * (k - 1);
                A(ut, ijk) = 0.5 * (A(u, ijk) + A(u, ijk + 1));
                A(vt, ijk) = 0.5 * (A(v, ijk) + A(v, ijk + jo));
                A(wt, ijk) = 0.5 * (A(w, ijk) + A(w, ijk + ko));
            }
    for (int k = 2; k <= nk; k++)
        for (int j = 2; j <= nj; j++) {
            long ijk = 1 + jo * (j - 1) + ko * (k - 1);
            long ijke = ijk + 1, ijkn = ijk + jo, ijkne = ijkn + 1, ijkr = ijk + ko, ijkre = ijkr + 1;
            A(ut, ijk) = A(u, ijke);
            A(vt, ijk) = 0.25 * (A(v, ijk) + A(v, ijke) + A(v, ijkn) + A(v, ijkne));
            A(wt, ijk) = 0.25 * (A(w, ijk) + A(w, ijke) + A(w, ijkr) + A(w, ijkre));
            ijk = nip1 + jo * (j - 1) + ko * (k - 1);
            long ijkw = ijk - 1, ijknw;
            ijkn = ijk + jo;
            ijknw = ijkn - 1;
            ijkr = ijk + ko;
            long ijkrw = ijkr - 1;
            A(ut, ijk) = A(u, ijk);
            A(vt, ijk) = 0.25 * (A(v, ijk) + A(v, ijkw) + A(v, ijkn) + A(v, ijknw));
            A(wt, ijk) = 0.25 * (A(w, ijk) + A(w, ijkw) + A(w, ijkr) + A(w, ijkrw));
        }
    for (int i = 2; i <= ni; i++)
        for (int j = 2; j <= nj; j++) {
            long ijk = i + jo * (j - 1);
            long ijkr = ijk + ko, ijkn = ijk + jo, ijknr = ijkn + ko, ijke = ijk + 1, ijkre = ijkr + 1;
            A(wt, ijk) = A(w, ijkr);
            A(vt, ijk) = 0.25 * (A(v, ijk) + A(v, ijkr) + A(v, ijkn) + A(v, ijknr));
            A(ut, ijk) = 0.25 * (A(u, ijk) + A(u, ijkr) + A(u, ijke) + A(u, ijkre));
            ijk = i + jo * (j - 1) + ko * (nkp1 - 1);
            long ijkl = ijk - ko, ijknl, ijkle;
            ijkn = ijk + jo;
            ijknl = ijkn - ko;
            ijke = ijk + 1;
            ijkle = ijkl + 1;
            A(wt, ijk) = A(w, ijk);
            A(vt, ijk) = 0.25 * (A(v, ijk) + A(v, ijkl) + A(v, ijkn) + A(v, ijknl));
            A(ut, ijk) = 0.25 * (A(u, ijk) + A(u, ijkl) + A(u, ijke) + A(u, ijkle));
        }
    for (int k = 2; k <= nk; k++)
        for (int i = 2; i <= ni; i++) {
            long ijk = i + ko * (k - 1);
            long ijkn = ijk + jo, ijkr = ijk + ko, ijknr = ijkr + jo, ijke = ijk + 1, ijkne = ijkn + 1;
            A(vt, ijk) = A(v, ijkn);
            A(wt, ijk) = 0.25 * (A(w, ijk) + A(w, ijkn) + A(w, ijkr) + A(w, ijknr));
            A(ut, ijk) = 0.25 * (A(u, ijk) + A(u, ijkn) + A(u, ijke) + A(u, ijkne));
            ijk = i + jo * (njp1 - 1) + ko * (k - 1);
            long ijks = ijk - jo, ijksr, ijkse;
            ijkr = ijk + ko;
            ijksr = ijkr - jo;
            ijke = ijk + 1;
            ijkse = ijks + 1;
            A(vt, ijk) = A(v, ijk);
            A(wt, ijk) = 0.25 * (A(w, ijk) + A(w, ijks) + A(w, ijkr) + A(w, ijksr));
            A(ut, ijk) = 0.25 * (A(u, ijk) + A(u, ijks) + A(u, ijke) + A(u, ijkse));
        }
}

/* outs (2-D, level-1 metric layout): um vm wm pm rhom ruv rvw rwu ruu rvv
 * rww rrh fm rff sc1varm T_m */
void orc_statistics(orc_ctx *c, int no_sam, const double *u, const double *v, const double *w, const double *p,
                    const double *rho, const double *sc1, const double *sc1var, const double *gam,
                    double *const *outs)
{
    for (int b = 1; b <= c->numbl; b++) {
        const int *n = c->mg_nijkp1[1][b];
        int nip1 = n[0], njp1 = n[1], nkp1 = n[2];
        long o3 = c->off3[1][b], o2 = c->off2[1][b], np = (long)nip1 * njp1 * nkp1;
        double *ut = (double *)calloc((size_t)np, sizeof(double));
        double *vt = (double *)calloc((size_t)np, sizeof(double));
        double *wt = (double *)calloc((size_t)np, sizeof(double));
        centre(nip1, njp1, nkp1, u + o3, v + o3, w + o3, ut, vt, wt);
        const double *r = rho + o3;
        long jo = nip1, ko = (long)nip1 * njp1;
        for (int j = 1; j <= njp1; j++)
            for (int i = 1; i <= nip1; i++) {
                double s[16] = {0};
                for (int k = 2; k <= nkp1 - 1; k++) {
                    long ijk = i + jo * (j - 1) + ko * (k - 1);
                    double rr = A(r, ijk), uu = A(ut, ijk), vv = A(vt, ijk), ww = A(wt, ijk);
                    s[0] = s[0] + rr * uu;
                    s[1] = s[1] + rr * vv;
                    s[2] = s[2] + rr * ww;
                    s[3] = s[3] + A(p + o3, ijk);
                    s[4] = s[4] + rr;
                    s[5] = s[5] + rr * uu * vv;
                    s[6] = s[6] + rr * vv * ww;
                    s[7] = s[7] + rr * uu * ww;
                    s[8] = s[8] + rr * uu * uu;
                    s[9] = s[9] + rr * vv * vv;
                    s[10] = s[10] + rr * ww * ww;
                    s[11] = s[11] + rr * rr;
                    s[12] = s[12] + A(sc1 + o3, ijk);
                    s[13] = s[13] + A(sc1 + o3, ijk) * A(sc1 + o3, ijk);
                    s[14] = s[14] + A(sc1var + o3, ijk);
                    s[15] = s[15] + A(gam + o3, ijk);
                }
                long ij = o2 + i + (long)nip1 * (j - 1);
                for (int q = 0; q < 16; q++) {
                    double avg = s[q] / (double)(nkp1 - 2);
                    A(outs[q], ij) = (A(outs[q], ij) * (double)(no_sam - 1) + avg) / (double)no_sam;
                }
            }
        free(ut);
        free(vt);
        free(wt);
    }
}
