/*
 * orc_outflow.c -- oracle: convective outflow and fixed inflow sides.
 * TEST INFRASTRUCTURE ONLY.
 *
 *   conv_exitbc          code/conv_exitbc.F:21-607 (tasks 1 and 2, with the
 *                        SAVEd side totals and inflow/outflow sums)
 *   conv_exitbc1_block   code/conv_exitbc1_block.F:6-133
 *   conv_exitbc2_block   code/conv_exitbc2_block.F:6-104
 *   conv_exitbc_scale    code/conv_exitbc_scale.F:6-70
 *   mass_flux            code/mass_flux.F:6-102
 *   mass_change          code/mass_change.F:6-83, mass_change_block.F:6-69
 *   fixed_inlet          code/fixed_inlet.F:5-180
 *
 * MPI_ALLREDUCE sums become sums over the blocks in block order.  The
 * conv_exitbc_scale call reaches v_int and w_int through an arena offset
 * from u_int (conv_exitbc.F:580); here the three arrays are passed.
 *
 * fixed_inlet draws its perturbations from the Fortran intrinsic
 * random_number, whose generator is the compiler's; this restatement uses a
 * counter-based generator instead (the splitmix64 finaliser of a key made
 * from the seed, the step, the block and the point), so the perturbations
 * differ from any particular Fortran build by construction.  The draw that
 * the reference overwrites (fixed_inlet.F:90-93) is not made.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include "orc_internal.h"

enum { M_DIP, M_DIU, M_DIV, M_DIX, M_RDIP, M_RDIV, M_RDIX, M_DJP, M_DJU, M_DJV, M_DJX, M_RDJP,
       M_RDJU, M_RDJX, M_HIJP, M_HJIP, M_HKIP, M_HKJP, M_HIJU, M_HJIU, M_HKIU, M_HKJU, M_HIJV,
       M_HJIV, M_HKIV, M_HKJV, M_RP, M_RU, M_RV, M_DIDJP, M_RDIDJP, M_DIDJU, M_RDIDJU, M_DJDIV,
       M_RDJDIV };

static int per_or_int(int bc) { return bc == ORC_BCT_PERIODIC || bc == ORC_BCT_INTERFACE; }

/* set_loop_bound(ivar, 1, 1, iblk, iblk, 1, ijkse) at level 1 (code/set_loop_bound.F:65-82) */
static void bounds(const orc_ctx *c, int b, int ivar, int se[6])
{
    const int *n = c->mg_nijkp1[1][b], *bcb = c->bl_bc[b];
    se[0] = (ivar == ORC_SV_U && !per_or_int(bcb[0])) ? 3 : 2;
    se[1] = n[0] - 1;
    se[2] = (ivar == ORC_SV_V && !per_or_int(bcb[2])) ? 3 : 2;
    se[3] = n[1] - 1;
    se[4] = (ivar == ORC_SV_W && !per_or_int(bcb[4])) ? 3 : 2;
    se[5] = n[2] - 1;
}

/* code/mass_flux.F:6-102 on one block (arrays offset to the block) */
static void mass_flux(int plane, int nip1, int njp1, int d1, int iva, const int se[6],
                      double *area, double *area_rho, double *mflux, const double *u,
                      const double *v, const double *w, const double *rho, const double *rdju,
                      const double *rdiv, const double *didjp, const double *dkp)
{
    *area = 0.;
    *mflux = 0.;
    *area_rho = 0.;
    if (d1 != iva) return;
    long jo = nip1, ko = (long)nip1 * njp1;
    if (d1 == ORC_SV_U) {
        for (int k = se[4]; k <= se[5]; k++) {
            long ikoff = ko * (k - 1) + plane;
            for (int j = se[2]; j <= se[3]; j++) {
                long ijk = jo * (j - 1) + ikoff;
                double areaf = A(rdju, plane + jo * (j - 1)) * A(dkp, k);
                *area = *area + areaf;
                *mflux = *mflux + 0.5 * (A(rho, ijk) + A(rho, ijk - 1)) * A(u, ijk) * areaf;
                *area_rho = *area_rho + 0.5 * (A(rho, ijk) + A(rho, ijk - 1)) * areaf;
            }
        }
    } else if (d1 == ORC_SV_V) {
        long joff = jo * (plane - 1);
        for (int k = se[4]; k <= se[5]; k++) {
            long jkoff = ko * (k - 1) + joff;
            for (int i = se[0]; i <= se[1]; i++) {
                long ijk = i + jkoff;
                double areaf = A(rdiv, i + joff) * A(dkp, k);
                *area = *area + areaf;
                *mflux = *mflux + 0.5 * (A(rho, ijk) + A(rho, ijk - jo)) * A(v, ijk) * areaf;
                *area_rho = *area_rho + 0.5 * (A(rho, ijk) + A(rho, ijk - jo)) * areaf;
            }
        }
    } else {
        long koff = ko * (plane - 1);
        for (int j = se[2]; j <= se[3]; j++) {
            long joff = jo * (j - 1), jkoff = joff + koff;
            for (int i = se[0]; i <= se[1]; i++) {
                long ijk = i + jkoff;
                double areaf = A(didjp, i + joff);
                *area = *area + areaf;
                *mflux = *mflux + 0.5 * (A(rho, ijk) + A(rho, ijk - ko)) * A(w, ijk) * areaf;
                *area_rho = *area_rho + 0.5 * (A(rho, ijk) + A(rho, ijk - ko)) * areaf;
            }
        }
    }
}

/* the exit plane's index along d1 (conv_exitbc.F:141-143) */
static int exit_plane(int side, int d1, const int se[6])
{
    int mod_iside = side % 2;
    return (se[2 * d1 - 2] - 1) * mod_iside + (se[2 * d1 - 1] + 1) * (1 - mod_iside);
}

/* code/conv_exitbc1_block.F (task 1) or conv_exitbc2_block.F (task 2), in
 * the routine's own index roles (n1, n2, n3; strides io, jo, ko) */
static void exit_block(int task, int d1, int side, int nip1, const int r[6], long io, long jo,
                       long ko, double *u, double *u_int, const double *rho,
                       const double *rhonp1, double *hn, const double *dip, const double *rp,
                       const double *dkp, double dtime, double uave)
{
    double const1 = 1.5 * dtime, const2 = 0.5 * dtime;
    int istr = r[0], iend = r[1], jstr = r[2], jend = r[3], kstr = r[4], kend = r[5];
    if (d1 != ORC_SV_W) {
        int i, i1;
        long off, off2;
        double uave1;
        if (side % 2 == 1) {
            i = istr - 1;
            i1 = istr;
            off = -io;
            off2 = 0;
            uave1 = -uave;
        } else {
            i = iend + 1;
            i1 = iend;
            off = io;
            off2 = io;
            uave1 = uave;
        }
        long ioff3 = 1 + io * (i - 1), ioff2 = 1 + io * (i1 - 1);
        for (int k = kstr; k <= kend; k++) {
            long koff = ioff3 + ko * (k - 1);
            for (int j = jstr; j <= jend; j++) {
                long ijk = koff + jo * (j - 1), ijk2 = ijk - off2, ij = ioff2 + jo * (j - 1);
                if (task == 2) {
                    A(u, ijk) = A(u_int, ijk);
                    continue;
                }
                double rho1 = 0.5 * (A(rho, ijk2) + A(rho, ijk2 + off));
                double rho2 = 0.5 * (A(rho, ijk2) + A(rho, ijk2 - off));
                double h = uave1 * (rho1 * A(u, ijk) - rho2 * A(u, ijk - off)) / A(dip, ij);
                double rhonp1_1 = 0.5 * (A(rhonp1, ijk2) + A(rhonp1, ijk2 + off));
                A(u_int, ijk) = (rho1 * A(u, ijk) - const1 * h + const2 * A(hn, ijk)) / rhonp1_1;
                A(hn, ijk) = h;
            }
        }
    } else {
        int k, k1;
        long off, off2;
        double uave1;
        if (side % 2 == 1) {
            k = kstr - 1;
            k1 = kstr;
            off = -ko;
            off2 = 0;
            uave1 = -uave;
        } else {
            k = kend + 1;
            k1 = kend;
            off = ko;
            off2 = ko;
            uave1 = uave;
        }
        long koff = ko * (k - 1);
        for (int j = jstr; j <= jend; j++) {
            long joff = koff + jo * (j - 1);
            for (int i = istr; i <= iend; i++) {
                long ijk = i + joff, ijk2 = ijk - off2, ij = i + (long)nip1 * (j - 1);
                if (task == 2) {
                    A(u, ijk) = A(u_int, ijk);
                    continue;
                }
                double rho1 = 0.5 * (A(rho, ijk2) + A(rho, ijk2 + off));
                double rho2 = 0.5 * (A(rho, ijk2) + A(rho, ijk2 - off));
                double h = uave1 * (rho1 * A(u, ijk) - rho2 * A(u, ijk - off)) / (A(rp, ij) * A(dkp, k1));
                double rhonp1_1 = 0.5 * (A(rhonp1, ijk2) + A(rhonp1, ijk2 + off));
                A(u_int, ijk) = (rho1 * A(u, ijk) - const1 * h + const2 * A(hn, ijk)) / rhonp1_1;
                A(hn, ijk) = h;
            }
        }
    }
}

/* code/conv_exitbc_scale.F:6-70 */
static void exit_scale(const orc_ctx *c, int iva, int side, int b, double *u, double scalef)
{
    const int *n = c->mg_nijkp1[1][b];
    int d1 = (side + 1) / 2, d2 = ORC_CYC1(1, d1), d3 = ORC_CYC1(2, d1);
    long ijko[4] = {0, 1, n[0], (long)n[0] * n[1]};
    long io = ijko[d1], jo = ijko[d2], ko = ijko[d3];
    int se[6];
    bounds(c, b, iva, se);
    int istr = se[2 * d1 - 2], iend = se[2 * d1 - 1];
    int jstr = se[2 * d2 - 2], jend = se[2 * d2 - 1];
    int kstr = se[2 * d3 - 2], kend = se[2 * d3 - 1];
    int i = (side % 2 == 1) ? istr - 1 : iend + 1;
    long ioff = 1 + io * (i - 1);
    for (int k = kstr; k <= kend; k++) {
        long koff = ioff + ko * (k - 1);
        for (int j = jstr; j <= jend; j++) {
            long ijk = koff + jo * (j - 1);
            A(u, ijk) = A(u, ijk) * scalef;
        }
    }
}

double orc_mass_change(orc_ctx *c, double dtime, const double *rho, const double *rhonp1,
                       const double *rdidjp, const double *dkw)
{
    double mass_chg = 0.;
    for (int b = 1; b <= c->numbl; b++) {
        const int *n = c->mg_nijkp1[1][b];
        int nip1 = n[0], njp1 = n[1], nkp1 = n[2];
        const double *rb = rho + c->off3[1][b], *rn = rhonp1 + c->off3[1][b];
        const double *rv = rdidjp + c->off2[1][b], *dk = dkw + c->off1k[1][b];
        long jo = nip1, ko = (long)nip1 * njp1;
        double ddtime = 1.0 / dtime, blk = 0.;
        for (int k = 2; k <= nkp1 - 1; k++) {
            long koff = ko * (k - 1);
            for (int j = 2; j <= njp1 - 1; j++) {
                long jk = jo * (j - 1) + koff;
                for (int i = 2; i <= nip1 - 1; i++) {
                    long ijk = i + jk;
                    double vol = A2(rv, i, j, nip1) * A(dk, k);
                    double cell_change = ddtime * vol * (A(rn, ijk) - A(rb, ijk));
                    blk = blk + cell_change;
                }
            }
        }
        mass_chg = mass_chg + blk;
    }
    return mass_chg;
}

int orc_has_convective(const orc_ctx *c)
{
    for (int b = 1; b <= c->numbl; b++)
        for (int s = 0; s < 6; s++)
            if (c->bl_bc[b][s] == ORC_BCT_CONVECTIVE) return 1;
    return 0;
}

void orc_conv_exitbc(orc_ctx *c, int task, int iva, double dtime, const double *rho,
                     const double *rhonp1, double *u, double *v, double *w, double *u_int,
                     double *v_int, double *w_int, double *hu, double *hv, double *hw,
                     const double *metric, const double *dkp, const double *dkw)
{
    if (!orc_has_convective(c)) return;
    const long T2 = c->tot2;
#define MET(a) (metric + (long)(a) * T2)
    double *ttl = c->exit_mflux_ttl, *arho = c->exit_arho_ttl;
    if (task == 1 && iva == ORC_SV_U) {
        for (int s = 1; s <= 6; s++) ttl[s] = arho[s] = 0.;
        for (int b = 1; b <= c->numbl; b++)
            for (int s = 1; s <= 6; s++) {
                if (c->bl_bc[b][s - 1] != ORC_BCT_CONVECTIVE) continue;
                const int *n = c->mg_nijkp1[1][b];
                long p3 = c->off3[1][b], p2 = c->off2[1][b], p1 = c->off1k[1][b];
                int d1 = (s + 1) / 2, se[6];
                bounds(c, b, d1, se);
                int ip = exit_plane(s, d1, se);
                double area, area_rho, mflux;
                mass_flux(ip, n[0], n[1], d1, d1, se, &area, &area_rho, &mflux, u + p3, v + p3, w + p3,
                          rhonp1 + p3, MET(M_RDJU) + p2, MET(M_RDIV) + p2, MET(M_DIDJP) + p2, dkp + p1);
                ttl[s] = ttl[s] + mflux;
                arho[s] = arho[s] + area_rho;
            }
    }
    if (iva == ORC_SV_U) {
        c->exit_mflux_in = 0.;
        c->exit_mflux_out = 0.;
    }
    double *vel[4] = {0, u, v, w}, *vint[4] = {0, u_int, v_int, w_int}, *hn[4] = {0, hu, hv, hw};
    for (int b = 1; b <= c->numbl; b++)
        for (int s = 1; s <= 6; s++) {
            const int *n = c->mg_nijkp1[1][b];
            int nip1 = n[0], njp1 = n[1];
            long p3 = c->off3[1][b], p2 = c->off2[1][b], p1 = c->off1k[1][b];
            int d1 = (s + 1) / 2, se[6];
            bounds(c, b, d1, se);
            int ip = exit_plane(s, d1, se);
            const double *fu = task == 1 ? u_int : u, *fv = task == 1 ? v_int : v, *fw = task == 1 ? w_int : w;
            double area, area_rho, mflux;
            if (c->bl_bc[b][s - 1] == ORC_BCT_FIXED) {
                mass_flux(ip, nip1, njp1, d1, iva, se, &area, &area_rho, &mflux, fu + p3, fv + p3, fw + p3,
                          rhonp1 + p3, MET(M_RDJU) + p2, MET(M_RDIV) + p2, MET(M_DIDJP) + p2, dkp + p1);
                c->exit_mflux_in = c->exit_mflux_in + mflux;
            }
            if (c->bl_bc[b][s - 1] != ORC_BCT_CONVECTIVE) continue;
            double uave = ttl[s] / arho[s];
            int r[6];
            bounds(c, b, iva, r);
            if (iva >= ORC_SV_U && iva <= ORC_SV_W) {
                long io = 1, jo = nip1, ko = (long)nip1 * njp1;
                /* metric arguments of conv_exitbc.F:262-338 per (d1, iva) */
                const double *dm, *rm, *km;
                if (d1 == ORC_SV_U) {
                    dm = MET(iva == ORC_SV_U ? M_DIP : iva == ORC_SV_V ? M_DIX : M_DIU);
                    rm = MET(M_RP);
                    km = dkp;
                } else if (d1 == ORC_SV_V) {
                    dm = MET(iva == ORC_SV_U ? M_DJX : iva == ORC_SV_V ? M_DJP : M_DJV);
                    rm = MET(M_RP);
                    km = dkp;
                } else {
                    dm = MET(M_DJX);
                    rm = MET(iva == ORC_SV_U ? M_RU : iva == ORC_SV_V ? M_RV : M_RP);
                    km = iva == ORC_SV_W ? dkp : dkw;
                }
                double *uu = vel[iva] + p3, *ui = vint[iva] + p3, *hh = hn[iva] + p3;
                if (d1 == ORC_SV_V) {
                    int rs[6] = {r[2], r[3], r[0], r[1], r[4], r[5]};
                    exit_block(task, d1, s, njp1, rs, jo, io, ko, uu, ui, rho + p3, rhonp1 + p3, hh,
                               dm + p2, rm + p2, km + p1, dtime, uave);
                } else {
                    exit_block(task, d1, s, nip1, r, io, jo, ko, uu, ui, rho + p3, rhonp1 + p3, hh,
                               dm + p2, rm + p2, km + p1, dtime, uave);
                }
            }
            mass_flux(ip, nip1, njp1, d1, iva, r, &area, &area_rho, &mflux, fu + p3, fv + p3, fw + p3,
                      rhonp1 + p3, MET(M_RDJU) + p2, MET(M_RDIV) + p2, MET(M_DIDJP) + p2, dkp + p1);
            c->exit_mflux_out = c->exit_mflux_out + mflux;
        }
    if (iva == ORC_SV_W && task == 1) {
        double mchg = orc_mass_change(c, dtime, rho, rhonp1, MET(M_RDIDJP), dkw);
        for (int iva1 = ORC_SV_U; iva1 <= ORC_SV_W; iva1++)
            for (int b = 1; b <= c->numbl; b++)
                for (int s = 1; s <= 6; s++) {
                    if (c->bl_bc[b][s - 1] != ORC_BCT_CONVECTIVE) continue;
                    double scale_factor = (c->exit_mflux_in - mchg) / c->exit_mflux_out;
                    exit_scale(c, iva1, s, b, vint[iva1] + c->off3[1][b], scale_factor);
                }
    }
#undef MET
}

/* ---- fixed_inlet ------------------------------------------------------ */
static uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

double orc_inlet_uniform(unsigned long long seed, int step, int block, int j, int k)
{
    uint64_t key = seed;
    key = key * 0x9E3779B97F4A7C15ULL + (uint64_t)(uint32_t)step;
    key = key * 0x9E3779B97F4A7C15ULL + (uint64_t)(uint32_t)block;
    key = key * 0x9E3779B97F4A7C15ULL + (uint64_t)(uint32_t)j;
    key = key * 0x9E3779B97F4A7C15ULL + (uint64_t)(uint32_t)k;
    return (double)(mix64(key) >> 11) * (1.0 / 9007199254740992.0);
}

void orc_fixed_inlet(orc_ctx *c, const int inlet[4], const double *uprof, const double *vprof,
                     unsigned long long seed, int step, double rholo, double rhohi, double *u,
                     double *v, double *w, double *sc1, double *rho, double *u_int, double *v_int,
                     double *w_int)
{
    for (int b = 1; b <= c->numbl; b++) {
        int which = 0;
        for (int q = 0; q < 4; q++)
            if (inlet[q] == b) which = q + 1;
        if (!which) continue;
        const int *n = c->mg_nijkp1[1][b];
        int nip1 = n[0], njp1 = n[1], nkp1 = n[2], nj = njp1 - 1;
        long jo = nip1, ko = (long)nip1 * njp1, boff3 = c->off3[1][b];
        for (int j = 1; j <= njp1; j++)
            for (int k = 1; k <= nkp1; k++) {
                double uin, vin, amp, fin, rhoin;
                int sh = (which - 1) * (nj - 1);
                uin = A(uprof, j + sh);
                vin = A(vprof, j + sh);
                amp = which <= 2 ? A(uprof, 3) : A(uprof, 4 * (nj - 2));
                fin = which <= 2 ? 0.0 : 1.0;
                rhoin = which <= 2 ? rholo : rhohi;
                double random = orc_inlet_uniform(seed, step, b, j, k);
                double perturb = 0.005 * amp * 2.0 * (random - 0.5);
                double win = perturb;
                uin = uin + perturb;
                vin = vin + perturb;
                long ijk = 2 + jo * (j - 1) + ko * (k - 1) + boff3, ijkw = ijk - 1;
                A(u, ijk) = uin;
                A(v, ijkw) = vin;
                A(w, ijkw) = win;
                A(sc1, ijkw) = fin;
                A(rho, ijkw) = rhoin;
                A(u_int, ijk) = A(u, ijk);
                A(v_int, ijkw) = A(v, ijkw);
                A(w_int, ijkw) = A(w, ijkw);
            }
    }
}

void orc_set_inlet(orc_ctx *c, const int inlet[4], const double *uprof, const double *vprof,
                   int nprof, unsigned long long seed)
{
    free(c->uprof);
    free(c->vprof);
    c->uprof = c->vprof = 0;
    for (int q = 0; q < 4; q++) c->inlet[q] = inlet ? inlet[q] : 0;
    c->inlet_seed = seed;
    if (nprof > 0) {
        c->uprof = (double *)malloc(sizeof(double) * nprof);
        c->vprof = (double *)malloc(sizeof(double) * nprof);
        for (int q = 0; q < nprof; q++) {
            c->uprof[q] = uprof[q];
            c->vprof[q] = vprof[q];
        }
    }
}

/* ---- recycling --------------------------------------------------------- */
/* mas-recyc/recycling.F:5-366 on the chain of blocks inblock..inblock+7
 * (1-based; those that exist), level 1.  The running means (umean ..
 * wwmean, indexed by j) and the target profiles (uprof .. wwprof) are
 * caller arrays; the reference's reads and writes of the means from and to
 * files (recycling.F:55-66, 148-156) are left to the caller.  jmult: 0 for
 * the inlet3 chain, njp1 - 2 for inlet2 (recycling.F:177-178), else 0.
 * rhohi is the density the recycled inflow plane takes. */
void orc_recycling(orc_ctx *c, int step, int inblock, const int inlet[4], double rhohi, double *u, double *v,
                   double *w, double *sc1, double *rho, double *u_int, double *v_int, double *w_int,
                   const double *uprof, const double *vprof, const double *wprof, const double *uuprof,
                   const double *vvprof, const double *wwprof, double *umean, double *vmean, double *wmean,
                   double *uumean, double *vvmean, double *wwmean)
{
    const double small = 0.0000001, cpfilt = 0.144;
    double *vel[3] = {u, v, w};
    double *mean[3] = {umean, vmean, wmean}, *rms[3] = {uumean, vvmean, wwmean};
    const double *prof[3] = {uprof, vprof, wprof}, *rprof[3] = {uuprof, vvprof, wwprof};
    for (int b = 1; b <= c->numbl; b++) {
        if (b < inblock || b > inblock + 7) continue;
        const int *n = c->mg_nijkp1[1][b];
        int nip1 = n[0], njp1 = n[1], nkp1 = n[2];
        long jo = nip1, ko = (long)nip1 * njp1, boff3 = c->off3[1][b];
        double *work = (double *)calloc((size_t)3 * (njp1 + 1) * (nkp1 + 1), sizeof(double));
#define WK(q, j, k) work[((size_t)(q) * (nkp1 + 1) + (k)) * (njp1 + 1) + (j)]
        for (int pass = 0; pass < 2; pass++) {
            for (int k = 2; k <= nkp1; k++) {
                long koff = (k - 1) * ko + boff3;
                for (int j = 2; j <= njp1; j++) {
                    long jkoff = (j - 1) * jo + koff;
                    for (int q = 0; q < 3; q++) {
                        double s = 0.0;
                        for (int i = 2; i <= nip1; i++) {
                            double d = A(vel[q], i + jkoff);
                            if (pass == 1) {
                                d = d - A(mean[q], j);
                                d = d * d;
                            }
                            s = s + d;
                        }
                        WK(q, j, k) = s / (double)(nip1 - 1);
                    }
                }
            }
            for (int j = 2; j <= njp1; j++)
                for (int q = 0; q < 3; q++) {
                    double s = 0.0;
                    for (int k = 2; k <= nkp1; k++) s = s + WK(q, j, k);
                    s = s / (double)(nkp1 - 1);
                    if (pass == 0)
                        A(mean[q], j) = cpfilt * s + (1. - cpfilt) * A(mean[q], j);
                    else
                        A(rms[q], j) = sqrt(cpfilt * s + (1. - cpfilt) * (A(rms[q], j) * A(rms[q], j)));
                }
        }
#undef WK
        free(work);
    }
    double *utemp = 0, *vtemp = 0, *wtemp = 0;
    long ntemp = 0;
    for (int b = 1; b <= c->numbl; b++) {
        const int *n = c->mg_nijkp1[1][b];
        int nip1 = n[0], njp1 = n[1], nkp1 = n[2];
        long jo = nip1, ko = (long)nip1 * njp1, boff3 = c->off3[1][b];
        if (step % 100 == 0 && step >= 200 && b >= inblock && b <= inblock + 7) {
            int jmult = 0;
            if (inblock == inlet[2]) jmult = 0;
            if (inblock == inlet[1]) jmult = njp1 - 2;
            for (int k = 2; k <= nkp1; k++) {
                long koff = (k - 1) * ko + boff3;
                for (int j = 2; j <= njp1; j++) {
                    long jkoff = (j - 1) * jo + koff;
                    for (int i = (b != inblock) ? 1 : 2; i <= nip1; i++) {
                        long ijk = i + jkoff;
                        for (int q = 0; q < 3; q++)
                            A(vel[q], ijk) = (A(rprof[q], j + jmult) / (A(rms[q], j) + small)) *
                                                 (A(vel[q], ijk) - A(mean[q], j)) +
                                             A(prof[q], j + jmult);
                    }
                }
            }
        }
        if (b == inblock + 7) {
            ntemp = (long)(njp1 - 1) * (nkp1 - 1);
            utemp = (double *)malloc(sizeof(double) * ntemp);
            vtemp = (double *)malloc(sizeof(double) * ntemp);
            wtemp = (double *)malloc(sizeof(double) * ntemp);
            long jk = 0;
            for (int k = 2; k <= nkp1; k++)
                for (int j = 2; j <= njp1; j++) {
                    long ijk = 3 + (j - 1) * jo + (k - 1) * ko + boff3, ijkw = ijk - 1;
                    utemp[jk] = A(u, ijk);
                    vtemp[jk] = A(v, ijkw);
                    wtemp[jk] = A(w, ijkw);
                    jk++;
                }
        }
    }
    if (utemp) {
        for (int b = 1; b <= c->numbl; b++) {
            if (b != inblock) continue;
            const int *n = c->mg_nijkp1[1][b];
            int nip1 = n[0], njp1 = n[1], nkp1 = n[2];
            long jo = nip1, ko = (long)nip1 * njp1, boff3 = c->off3[1][b];
            long jk = 0;
            for (int k = 2; k <= nkp1; k++)
                for (int j = 2; j <= njp1 && jk < ntemp; j++) {
                    long ijk = 2 + (j - 1) * jo + (k - 1) * ko + boff3, ijkw = ijk - 1;
                    A(u, ijk) = utemp[jk];
                    A(v, ijkw) = vtemp[jk];
                    A(w, ijkw) = wtemp[jk];
                    A(sc1, ijkw) = 1.0;
                    A(rho, ijkw) = rhohi;
                    A(u_int, ijk) = A(u, ijk);
                    A(v_int, ijkw) = A(v, ijkw);
                    A(w_int, ijkw) = A(w, ijkw);
                    jk++;
                }
        }
        free(utemp);
        free(vtemp);
        free(wtemp);
    }
}
