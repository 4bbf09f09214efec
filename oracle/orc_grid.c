/*
 * orc_grid.c -- oracle: block/level bookkeeping, loop bounds and the block
 * halo exchange.  TEST INFRASTRUCTURE ONLY (see lester_oracle.h).
 *
 * Restates, single process (one MPI rank owning every block):
 *   set_const    code/set_const.F:16-28       (cyclic, cyclic1)
 *   set_offset   code/set_offset.F:8-263      (levels, offsets, mult)
 *   set_interfaces code/set_interfaces.F:6-256 (face tables)
 *   set_loop_bound code/set_loop_bound.F:11-125
 *   swap_sc      code/swap_sc0.F:6-293        (pack all, then unpack all)
 */
#include <stdlib.h>
#include <string.h>
#include "orc_internal.h"

/* code/set_const.F:16-28 */
const int orc_cyclic[2][4] = {{0, 2, 3, 1}, {0, 3, 1, 2}};
const int orc_cyclic1[2][4] = {{0, 2, 1, 1}, {0, 3, 3, 2}};

/* code/set_offset.F:8-263.  nummgl_req = 0 means "use what is found". */
static int set_offset(orc_ctx *c, int nummgl_req)
{
    int numbl = c->numbl;
    int found = 1; /* set_offset.F leaves it unset when level 1 cannot coarsen */
    for (int b = 1; b <= numbl; b++)
        for (int d = 0; d < 3; d++) c->mg_nijkp1[1][b][d] = c->bl_nijkp1[b][d];

    /* set_offset.F:94-132: a coarser level exists only if every block can
     * halve on every axis and stays >= 4 points including ghosts */
    for (int lev = 1; lev <= c->maxmgl - 1; lev++) {
        int coarser = 1;
        for (int b = 1; b <= numbl; b++) {
            int *n = c->mg_nijkp1[lev][b];
            if (n[0] % 2 == 0 && n[1] % 2 == 0 && n[2] % 2 == 0 && coarser) {
                int ni = n[0] / 2 + 1, nj = n[1] / 2 + 1, nk = n[2] / 2 + 1;
                if (ni >= 4 && nj >= 4 && nk >= 4) {
                    c->mg_nijkp1[lev + 1][b][0] = ni;
                    c->mg_nijkp1[lev + 1][b][1] = nj;
                    c->mg_nijkp1[lev + 1][b][2] = nk;
                } else {
                    coarser = 0;
                }
            } else {
                coarser = 0;
            }
        }
        if (coarser)
            found = lev + 1;
        else
            break;
    }
    if (nummgl_req == 0)
        c->nummgl = found;
    else if (nummgl_req <= found)
        c->nummgl = nummgl_req;
    else
        return -1; /* set_offset.F:149-151 stops */

    /* offsets: a running total over (level, block) -- set_offset.F:166-234 */
    long o3 = 0, o2 = 0, o1 = 0, oxy = 0, oz = 0, oki = 0, ojk = 0;
    for (int lev = 1; lev <= c->nummgl; lev++) {
        for (int b = 1; b <= numbl; b++) {
            int *n = c->mg_nijkp1[lev][b];
            c->off3[lev][b] = o3;
            c->off2[lev][b] = o2;
            c->off1k[lev][b] = o1;
            c->offxy[lev][b] = oxy;
            c->offz[lev][b] = oz;
            c->offki[lev][b] = oki;
            c->offjk[lev][b] = ojk;
            o3 += (long)n[0] * n[1] * n[2];
            o2 += (long)n[0] * n[1];
            o1 += n[2];
            oxy += (long)(n[0] + 1) * (n[1] + 1);
            oz += n[2] + 1;
            oki += (long)n[2] * n[0];
            ojk += (long)n[1] * n[2];
        }
        if (lev == 1) {
            c->tot_sg3 = o3;
            c->tot_ki = oki;
            c->tot_jk = ojk;
        }
    }
    c->tot3 = o3;
    c->tot2 = o2;
    c->tot1k = o1;
    c->totxy = oxy;
    c->totz = oz;

    /* set_offset.F:242-260 */
    for (int lev = 1; lev <= c->nummgl - 1; lev++)
        for (int b = 1; b <= numbl; b++)
            for (int d = 0; d < 3; d++)
                c->mult[lev][b][d] =
                    (c->mg_nijkp1[lev][b][d] == c->mg_nijkp1[lev + 1][b][d]) ? 1 : 2;
    return 0;
}

/* code/set_interfaces.F:115-203, one rank */
static int set_interfaces(orc_ctx *c)
{
    for (int ig = 1; ig <= c->nummgl; ig++) {
        long i1 = 1;
        for (int b = 1; b <= c->numbl; b++) {
            for (int s = 1; s <= 6; s++) {
                int bn = c->bl2bl[b][s - 1];
                int sn = c->bl2side[b][s - 1];
                if (bn == 0) continue;
                if ((s % 2) == (sn % 2)) return -2; /* set_interfaces.F:416-422 */
                int d1 = (s + 1) / 2;
                int d2 = ORC_CYC(1, d1), d3 = ORC_CYC(2, d1);
                int *n = c->mg_nijkp1[ig][b];
                int nip1 = n[d1 - 1], njp1 = n[d2 - 1], nkp1 = n[d3 - 1];
                long ijko[4] = {0, 1, n[0], (long)n[0] * n[1]};
                long io = ijko[d1], jo = ijko[d2], ko = ijko[d3];
                long p31 = c->off3[ig][b];
                long p32 = c->off3[1][b]; /* sg_off == level-1 mg_off */
                int i, i2;
                if (s % 2 == 0) { i = nip1 - 1; i2 = nip1; }
                else { i = 2; i2 = 1; }
                long *ik = c->inikoff[ig][b][s - 1];
                ik[0] = 1 + io * (i - 1) + p31;
                ik[1] = 1 + io * (i - 1) + p32;
                ik[2] = 1 + io * (i2 - 1) + p31;
                ik[3] = 1 + io * (i2 - 1) + p32;
                ik[4] = jo;
                ik[5] = ko;
                c->inwoff[ig][b][s - 1] = i1;
                c->iniknum[ig][b][s - 1][0] = njp1;
                c->iniknum[ig][b][s - 1][1] = nkp1;
                i1 += (long)njp1 * nkp1 + 1;
            }
        }
        c->inoffmax[ig] = i1 + 1;
        if (i1 + 1 > c->lwork) c->lwork = i1 + 1;
    }
    /* partner faces must agree in size (set_interfaces.F:477-481) */
    for (int ig = 1; ig <= c->nummgl; ig++)
        for (int b = 1; b <= c->numbl; b++)
            for (int s = 1; s <= 6; s++) {
                int bn = c->bl2bl[b][s - 1], sn = c->bl2side[b][s - 1];
                if (bn == 0) continue;
                if (c->iniknum[ig][b][s - 1][0] != c->iniknum[ig][bn][sn - 1][0] ||
                    c->iniknum[ig][b][s - 1][1] != c->iniknum[ig][bn][sn - 1][1])
                    return -3;
            }
    return 0;
}

orc_ctx *orc_create(int numbl, const int *nijkp1, const int *bc,
                    const int *bl2bl, const int *bl2side, int maxmgl,
                    int nummgl_req, int *status)
{
    *status = 0;
    if (numbl < 1 || numbl > ORC_MAXBL || maxmgl < 1 || maxmgl > ORC_MAXMGL) {
        *status = -10;
        return NULL;
    }
    orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
    c->numbl = numbl;
    c->maxmgl = maxmgl;
    for (int b = 1; b <= numbl; b++) {
        for (int d = 0; d < 3; d++) c->bl_nijkp1[b][d] = nijkp1[(b - 1) * 3 + d];
        for (int s = 0; s < 6; s++) {
            c->bl_bc[b][s] = bc[(b - 1) * 6 + s];
            c->bl2bl[b][s] = bl2bl[(b - 1) * 6 + s];
            c->bl2side[b][s] = bl2side[(b - 1) * 6 + s];
            int t = c->bl_bc[b][s];
            if ((t == ORC_BCT_PERIODIC || t == ORC_BCT_INTERFACE) && c->bl2bl[b][s] == 0) {
                *status = -4;
                free(c);
                return NULL;
            }
        }
    }
    int st = set_offset(c, nummgl_req);
    if (st == 0) st = set_interfaces(c);
    if (st != 0) {
        *status = st;
        free(c);
        return NULL;
    }
    c->work = (double *)calloc((size_t)c->lwork + 1, sizeof(double));
    orc_set_loop_bound(c, ORC_SV_P);
    return c;
}

void orc_destroy(orc_ctx *c)
{
    if (!c) return;
    free(c->work);
    free(c->uprof);
    free(c->vprof);
    free(c);
}

void orc_sizes(const orc_ctx *c, long *out)
{
    out[0] = c->nummgl;
    out[1] = c->tot3;
    out[2] = c->tot_sg3;
    out[3] = c->tot2;
    out[4] = c->tot1k;
    out[5] = c->totxy;
    out[6] = c->totz;
    out[7] = c->tot_ki;
    out[8] = c->tot_jk;
}

void orc_block_info(const orc_ctx *c, int ilev, int iblk, int *nijk, int *mult,
                    long *offs)
{
    for (int d = 0; d < 3; d++) {
        nijk[d] = c->mg_nijkp1[ilev][iblk][d];
        mult[d] = c->mult[ilev][iblk][d];
    }
    offs[0] = c->off3[ilev][iblk];
    offs[1] = c->off2[ilev][iblk];
    offs[2] = c->off1k[ilev][iblk];
    offs[3] = c->offxy[ilev][iblk];
    offs[4] = c->offz[ilev][iblk];
    offs[5] = c->offki[ilev][iblk];
    offs[6] = c->offjk[ilev][iblk];
}

/* code/set_loop_bound.F:316-385 with choice = 2, all levels and blocks */
void orc_set_loop_bound(orc_ctx *c, int ivar)
{
    for (int lev = 1; lev <= c->nummgl; lev++) {
        double npts = 0;
        for (int b = 1; b <= c->numbl; b++) {
            int *n = c->mg_nijkp1[lev][b];
            int *bcb = c->bl_bc[b];
            int istr = (ivar == ORC_SV_U && bcb[0] != ORC_BCT_PERIODIC && bcb[0] != ORC_BCT_INTERFACE) ? 3 : 2;
            int jstr = (ivar == ORC_SV_V && bcb[2] != ORC_BCT_PERIODIC && bcb[2] != ORC_BCT_INTERFACE) ? 3 : 2;
            int kstr = (ivar == ORC_SV_W && bcb[4] != ORC_BCT_PERIODIC && bcb[4] != ORC_BCT_INTERFACE) ? 3 : 2;
            int *se = c->nijkse[lev][b];
            se[0] = istr;
            se[1] = n[0] - 1;
            se[2] = jstr;
            se[3] = n[1] - 1;
            se[4] = kstr;
            se[5] = n[2] - 1;
            npts = npts + (double)(n[0] - istr) * (double)(n[1] - jstr) * (double)(n[2] - kstr);
        }
        c->npts_all[lev] = npts;
    }
}

double orc_npts_all(const orc_ctx *c, int ilev) { return c->npts_all[ilev]; }
void orc_set_jumble(orc_ctx *c, int jumble) { c->jumble = jumble; }
int orc_get_jumble(const orc_ctx *c) { return c->jumble; }

/* code/swap_sc0.F:6-293, one rank: every face is packed into work before any
 * ghost plane is written, so edges and corners see the pre-exchange state. */
void orc_swap_sc(orc_ctx *c, int ig, double *var, int mg_or_sg)
{
    double *work = c->work;
    for (int b = 1; b <= c->numbl; b++)
        for (int s = 1; s <= 6; s++) {
            int t = c->bl_bc[b][s - 1];
            if (t != ORC_BCT_INTERFACE && t != ORC_BCT_PERIODIC) continue;
            long *ik = c->inikoff[ig][b][s - 1];
            int nj = c->iniknum[ig][b][s - 1][0], nk = c->iniknum[ig][b][s - 1][1];
            long ioff = (mg_or_sg == 1) ? ik[0] : ik[1];
            long jo = ik[4], ko = ik[5];
            long i1 = c->inwoff[ig][b][s - 1];
            for (int k = 1; k <= nk; k++) {
                long ikoff = ko * (k - 1) + ioff;
                for (int j = 1; j <= nj; j++) {
                    A(work, i1) = A(var, ikoff + jo * (j - 1));
                    i1++;
                }
            }
        }
    for (int b = 1; b <= c->numbl; b++)
        for (int s = 1; s <= 6; s++) {
            int t = c->bl_bc[b][s - 1];
            if (t != ORC_BCT_INTERFACE && t != ORC_BCT_PERIODIC) continue;
            int bn = c->bl2bl[b][s - 1], sn = c->bl2side[b][s - 1];
            if (bn == 0) continue;
            long *ik = c->inikoff[ig][b][s - 1];
            int nj = c->iniknum[ig][b][s - 1][0], nk = c->iniknum[ig][b][s - 1][1];
            long ioff = (mg_or_sg == 1) ? ik[2] : ik[3];
            long jo = ik[4], ko = ik[5];
            long i1 = c->inwoff[ig][bn][sn - 1];
            for (int k = 1; k <= nk; k++) {
                long ikoff = ko * (k - 1) + ioff;
                for (int j = 1; j <= nj; j++) {
                    A(var, ikoff + jo * (j - 1)) = A(work, i1);
                    i1++;
                }
            }
        }
}
