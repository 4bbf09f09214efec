/*
 * orc_step.c -- oracle: one time step in the order of code/step.F:214-454.
 * TEST INFRASTRUCTURE ONLY.
 *
 * ivar = u: fixed_inlet on the inlet blocks (step.F:226), set_virt_bc for
 *   u, v, w (236-255), subgrid (258),
 *   set_gamsc1_bc, set_sc1, set_sc1_bc, set_sc1var, search_lib, set_sc1_bc
 *   x3 (268-298), set_uv_int(u) (307), conv_exitbc(1, u) (344)
 * ivar = v: set_uv_int with the v arrays in the u roles (319-326),
 *   conv_exitbc(1, v)
 * ivar = w: set_w_int (331), conv_exitbc(1, w)
 * ivar = p: coeff_p at istep 1 (359-362), sour_p (366), lmg_solve (372),
 *   extrap_p (376), p_ref_subtract (380), uvw_adv x3 (418-425), slipbc
 *   (428), conv_exitbc(2, u..w) (433-441), swap_rhos (450)
 * conv_exitbc is a no-op without convective sides; conv_exitbc(1, p) and
 * (1, sc1) change nothing; cflest only prints.
 * With mg->compat (not in the reference) the pressure source loses its
 * interior mean before lmg_solve: the compatible system of a singular
 * (all-Neumann/periodic) pressure equation, solved to tolf, is the FP64
 * reference for the GPU fast solvers on variable-density cases.
 */
#include <stdlib.h>
#include "orc_internal.h"

void orc_set_virt_bc(orc_ctx *c, int iva, double visc, double kappa, double aplus,
                     double ylaminar, double *f, const double *rho, double *vdd,
                     const double *metric, const double *dkp, const double *dkw,
                     double *const *tw);

enum { M_DIP, M_DIU, M_DIV, M_DIX, M_RDIP, M_RDIV, M_RDIX, M_DJP, M_DJU, M_DJV, M_DJX, M_RDJP,
       M_RDJU, M_RDJX, M_HIJP, M_HJIP, M_HKIP, M_HKJP, M_HIJU, M_HJIU, M_HKIU, M_HKJU, M_HIJV,
       M_HJIV, M_HKIV, M_HKJV, M_RP, M_RU, M_RV, M_DIDJP, M_RDIDJP, M_DIDJU, M_RDIDJU, M_DJDIV,
       M_RDJDIV };

void orc_step(orc_ctx *c, const orc_mgctrl *mg, const orc_phys *k, int istep, int iststep,
              orc_fields *F)
{
    double *metric = F->metric;
    long T2 = c->tot2;
#define MET(a) (metric + (long)(a) * T2)
    double *twu[4] = {F->tw[0], F->tw[1], F->tw[2], F->tw[3]};
    double *twv[4] = {F->tw[4], F->tw[5], F->tw[6], F->tw[7]};
    double *tww[4] = {F->tw[8], F->tw[9], F->tw[10], F->tw[11]};
    if (c->inlet[0] || c->inlet[1] || c->inlet[2] || c->inlet[3])
        orc_fixed_inlet(c, c->inlet, c->uprof, c->vprof, c->inlet_seed, istep, k->rholo, k->rhohi,
                        F->u, F->v, F->w, F->sc1, F->rho, F->u_int, F->v_int, F->w_int);
    orc_set_virt_bc(c, ORC_SV_U, k->visc, k->kappa, k->aplus, k->ylaminar, F->u, F->rho,
                    F->vd_damping, metric, F->dkp, F->dkw, twu);
    orc_set_virt_bc(c, ORC_SV_V, k->visc, k->kappa, k->aplus, k->ylaminar, F->v, F->rho,
                    F->vd_damping, metric, F->dkp, F->dkw, twv);
    orc_set_virt_bc(c, ORC_SV_W, k->visc, k->kappa, k->aplus, k->ylaminar, F->w, F->rho,
                    F->vd_damping, metric, F->dkp, F->dkw, tww);
    orc_subgrid(c, k->model, k->csles, k->gotrad, k->alpha, F->gam, F->gamsc1, F->u, F->v, F->w, F->sc1,
                F->sc1var, F->sc1dis, F->vd_damping, MET(M_DIP), MET(M_DIU), MET(M_DJP),
                MET(M_DJV), F->dkp, F->dkw, MET(M_HIJP), MET(M_HJIP), MET(M_HKIP), MET(M_HKJP),
                MET(M_RP));
    orc_set_gamsc1_bc(c, k->visc, F->sc1, F->gamsc1, F->gamlam, metric, F->dkp);
    orc_set_sc1(c, k->dtime, metric, F->dkp, F->dkw, F->u, F->v, F->w, F->sc1, F->hn_sc1, F->rho,
                F->gamsc1, F->gamlam);
    orc_set_sc1_bc(c, F->sc1);
    orc_set_sc1var(c, F->sc1, F->sc1var, metric, F->dkp, F->dkw);
    orc_search_lib(c, F->sc1, F->rhonp1, k->alpha, F->rho, k->rholo, k->rhohi);
    orc_swap_sc(c, 1, F->temperature, 2); /* search_lib.F:335 */
    orc_set_sc1_bc(c, F->sc1);
    orc_set_sc1_bc(c, F->rhonp1);
    orc_set_sc1_bc(c, F->temperature);
    orc_set_uv_int(c, ORC_SV_U, k->dtime, iststep, k->visc, k->ylaminar, k->kappa, k->cwfun,
                   F->u, F->v, F->w, F->p, F->rho, F->rhonp1, F->gam, F->u_int, F->hn_u, metric,
                   F->dkp, F->dkw, F->tw[0], F->tw[1], F->tw[2], F->tw[3]);
    orc_conv_exitbc(c, 1, ORC_SV_U, k->dtime, F->rho, F->rhonp1, F->u, F->v, F->w, F->u_int,
                    F->v_int, F->w_int, F->hn_u, F->hn_v, F->hn_w, metric, F->dkp, F->dkw);
    orc_set_uv_int(c, ORC_SV_V, k->dtime, iststep, k->visc, k->ylaminar, k->kappa, k->cwfun,
                   F->v, F->u, F->w, F->p, F->rho, F->rhonp1, F->gam, F->v_int, F->hn_v, metric,
                   F->dkp, F->dkw, F->tw[4], F->tw[5], F->tw[6], F->tw[7]);
    orc_conv_exitbc(c, 1, ORC_SV_V, k->dtime, F->rho, F->rhonp1, F->u, F->v, F->w, F->u_int,
                    F->v_int, F->w_int, F->hn_u, F->hn_v, F->hn_w, metric, F->dkp, F->dkw);
    orc_set_w_int(c, k->dtime, iststep, k->visc, k->ylaminar, k->kappa, k->cwfun, F->u, F->v,
                  F->w, F->p, F->rho, F->rhonp1, F->gam, F->w_int, F->hn_w, metric, F->dkp,
                  F->dkw, F->tw[10], F->tw[11], F->tw[8], F->tw[9]);
    orc_conv_exitbc(c, 1, ORC_SV_W, k->dtime, F->rho, F->rhonp1, F->u, F->v, F->w, F->u_int,
                    F->v_int, F->w_int, F->hn_u, F->hn_v, F->hn_w, metric, F->dkp, F->dkw);
    if (istep == 1)
        orc_coeff_p(c, MET(M_DIU), MET(M_DJV), MET(M_RDIV), MET(M_RDJU), MET(M_DIDJP), MET(M_RP),
                    F->dkp, F->dkw, F->ap, F->aw, F->ae, F->as, F->an, F->al, F->ar);
    orc_sour_p(c, k->dtime, MET(M_DIU), MET(M_DJV), MET(M_RDIV), MET(M_RDJU), MET(M_DIDJP),
               F->dkp, MET(M_RDIDJP), F->dkw, F->u_int, F->v_int, F->w_int, F->rho, F->rhonp1,
               F->drhonp1dt, F->s, F->srhot, F->srhoux);
    if (mg->compat) {
        /* interior mean, summed block by block in k, j, i order */
        double sum = 0.0, cnt = 0.0;
        for (int b = 1; b <= c->numbl; b++) {
            const int *n = c->mg_nijkp1[1][b];
            for (int k = 2; k <= n[2] - 1; k++)
                for (int j = 2; j <= n[1] - 1; j++)
                    for (int i = 2; i <= n[0] - 1; i++) {
                        sum += F->s[c->off3[1][b] + (i - 1) + (long)n[0] * ((j - 1) + (long)n[1] * (k - 1))];
                        cnt += 1.0;
                    }
        }
        const double mean = sum / cnt;
        for (int b = 1; b <= c->numbl; b++) {
            const int *n = c->mg_nijkp1[1][b];
            for (int k = 2; k <= n[2] - 1; k++)
                for (int j = 2; j <= n[1] - 1; j++)
                    for (int i = 2; i <= n[0] - 1; i++)
                        F->s[c->off3[1][b] + (i - 1) + (long)n[0] * ((j - 1) + (long)n[1] * (k - 1))] -= mean;
        }
    }
    orc_set_loop_bound(c, ORC_SV_P);
    double nrm[5];
    orc_lmg_solve(c, mg, F->ap, F->aw, F->ae, F->as, F->an, F->al, F->ar, F->p, F->s, F->res, nrm);
    orc_extrap_p(c, F->p);
    orc_p_ref_subtract(c, F->p);
    orc_uvw_adv(c, ORC_SV_U, k->dtime, MET(M_DIU), MET(M_RP), F->dkw, F->u, F->u_int, F->rhonp1, F->p);
    orc_uvw_adv(c, ORC_SV_V, k->dtime, MET(M_DJV), MET(M_RP), F->dkw, F->v, F->v_int, F->rhonp1, F->p);
    orc_uvw_adv(c, ORC_SV_W, k->dtime, MET(M_DIU), MET(M_RP), F->dkw, F->w, F->w_int, F->rhonp1, F->p);
    orc_slipbc(c, k->dtime, MET(M_DJP), F->u, F->v, F->v_int, F->w, F->sc1, F->rho, F->p);
    for (int iva = ORC_SV_U; iva <= ORC_SV_W; iva++)
        orc_conv_exitbc(c, 2, iva, k->dtime, F->rho, F->rhonp1, F->u, F->v, F->w, F->u_int,
                        F->v_int, F->w_int, F->hn_u, F->hn_v, F->hn_w, metric, F->dkp, F->dkw);
    orc_swap_rhos(c, F->rho, F->rhonp1, F->rhonm1);
#undef MET
}
