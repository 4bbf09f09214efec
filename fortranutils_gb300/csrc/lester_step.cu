// lester_step.cu -- one LES time step on the device: the ivar loop of
// code/step.F:214-454 (u, v, w, p; the sc1 pass has no work without a
// convective outflow) calling the library's routines in the reference's
// order.  Work the reference does only for output or diagnostics
// (statistics, field output, cflest) and the inflow/outflow routines of
// sides this library does not support (FIXED inlet, CONVECTIVE outflow)
// are not part of it; a block with such a side is refused.
//
// Field pointers may be host or device arrays.  Host arrays are copied to
// device mirrors before the step and back after it (one copy each way per
// call).  Scratch fields passed as NULL are kept on the device by the
// library.
#include <cstring>
#include "kernels.h"
#include "lester_ctx.h"

using namespace les;

extern "C" {

int lester_swap_sc(const int *, const int *, double *, double *, const int *);
int lester_coeff_p(const double *, const double *, const double *, const double *, const double *, const double *,
                   const double *, const double *, double *, double *, double *, double *, double *, double *,
                   double *);
int lester_sour_p(const double *, const double *, const double *, const double *, const double *, const double *,
                  const double *, const double *, const double *, const double *, const double *, const double *,
                  const double *, double *, double *, double *, double *, double *, double *);
int lester_lmg_solve(const double *, const double *, const double *, const double *, const double *,
                     const double *, const double *, double *, double *, double *, int *, double *);
int lester_extrap_p(double *, double *, int *);
int lester_p_ref_subtract(double *);
int lester_uvw_adv(const int *, const double *, const double *, const double *, double *, const double *,
                   const double *, const double *, double *, int *, const int *);
int lester_swap_rhos(double *, double *, double *);
int lester_search_lib(double *, double *, double *, double *, double *, int *, const int *, const double *,
                      const double *, const double *, const double *);
int lester_slipbc(const double *, const double *, const double *, const double *, const double *, const double *,
                  const double *, const double *, double *, double *, const double *, double *, double *, double *,
                  const double *, const int *);
int lester_subgrid(double *, double *, const double *, const double *, const double *, const double *,
                   const double *, double *, double *, const double *, const double *, const double *,
                   const double *, const double *, const double *, const double *, const double *, const double *,
                   const double *, const double *, const double *, double *, int *);
int lester_set_virt_bc(const int *, const int *, double *, const double *, const double *, const double *, double *,
                       int *, const double *, double *, double *, double *, double *, double *, double *, double *,
                       double *, double *, double *, double *, double *, const double *, const double *,
                       const double *, const double *, const double *, const double *, const double *,
                       const double *, const double *, const double *, const double *, const double *);
int lester_set_uv_int(const int *, const double *, const double *, const double *, const double *, const double *,
                      const double *, const double *, double *, double *, const double *, const double *,
                      const double *, const double *, const double *, const double *, const double *,
                      const double *, const double *, const double *, const double *, const double *,
                      const double *, const double *, const double *, const double *, const double *,
                      const double *, const double *, const double *, const double *, const double *, double *,
                      double *, double *, double *, double *, int *);
int lester_set_w_int(const double *, const double *, const double *, const double *, const double *,
                     const double *, const double *, double *, double *, const double *, const double *,
                     const double *, const double *, const double *, const double *, const double *,
                     const double *, const double *, const double *, const double *, const double *,
                     const double *, const double *, const double *, const double *, double *, double *, double *,
                     double *, double *, int *);
int lester_set_gamsc1_bc(const double *, double *, double *, const double *, const double *, const double *,
                         const double *);
int lester_set_sc1(const double *, const double *, const double *, const double *, double *, const double *,
                   const double *, const double *, double *, const double *, const double *, const double *,
                   const double *, const double *, const double *, const double *, const double *, const double *,
                   const double *, const double *, const double *, const double *, const double *, const double *,
                   double *, int *);
int lester_set_sc1_bc(double *);
int lester_set_sc1var(const double *, const double *, const double *, const double *, const double *, double *,
                      double *, const double *, const double *, const double *, const double *, const double *,
                      double *, int *);

#define RET(x)                                                                                     \
    do {                                                                                           \
        int rr_ = (x);                                                                             \
        if (rr_) return rr_;                                                                       \
    } while (0)

enum { M_DIP, M_DIU, M_DIV, M_DIX, M_RDIP, M_RDIV, M_RDIX, M_DJP, M_DJU, M_DJV, M_DJX, M_RDJP, M_RDJU,
       M_RDJX, M_HIJP, M_HJIP, M_HKIP, M_HKJP, M_HIJU, M_HJIU, M_HKIU, M_HKJU, M_HIJV, M_HJIV, M_HKIV,
       M_HKJV, M_RP, M_RU, M_RV, M_DIDJP, M_RDIDJP, M_DIDJU, M_RDIDJU, M_DJDIV, M_RDJDIV };

int lester_step(lester_fields *F, const int *istep)
{
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    if (!F || !istep) return set_err(LES_ERR_ARG, "null fields / istep");
    int r0;
    if ((r0 = ensure_sides(c))) return r0;
    if (has_inlet(c) && (!c.d_uprof || !c.d_vprof))
        return set_err(LES_ERR_ARG, "inlet blocks set without profiles (lester_gpu_set_inlet)");
    // whole-state staging: host arrays are mirrored once for the step
    Staging st(&c, __func__);
    lester_fields D = *F;
    long n3 = c.tot_sg3, nm = c.tot3;
    double **f3[] = {&D.u, &D.v, &D.w, &D.sc1, &D.rho, &D.rhonp1, &D.rhonm1, &D.u_int, &D.v_int, &D.w_int,
                     &D.hn_u, &D.hn_v, &D.hn_w, &D.hn_sc1, &D.gam, &D.gamsc1, &D.gamlam, &D.sc1var, &D.sc1dis,
                     &D.vd_damping, &D.temperature, &D.drhonp1dt, &D.srhot, &D.srhoux};
    int r;
    int nscr = 0;
    for (double **pp : f3) {
        if (*pp) RET(st.io(*pp, n3, pp));
        else {
            // library-held scratch field
            if ((int)c.scratch.size() <= nscr) {
                double *d = nullptr;
                if (cudaMalloc(&d, sizeof(double) * n3) != cudaSuccess) {
                    cudaGetLastError();
                    return set_err(LES_ERR_NOMEM, "step scratch allocation failed");
                }
                cudaMemsetAsync(d, 0, sizeof(double) * n3, c.stream);
                c.scratch.push_back(d);
            }
            *pp = c.scratch[nscr++];
        }
    }
    double **fm[] = {&D.p, &D.s, &D.res, &D.ap, &D.aw, &D.ae, &D.as, &D.an, &D.al, &D.ar};
    for (double **pp : fm) {
        if (!*pp) return set_err(LES_ERR_ARG, "p, s, res and the coefficient arrays are required");
        RET(st.io(*pp, nm, pp));
    }
    for (int q = 0; q < 35; q++) {
        if (!D.metric[q]) return set_err(LES_ERR_ARG, "metric %d missing", q);
        RET(st.io(D.metric[q], c.tot2, &D.metric[q]));
    }
    RET(st.io(D.dkp, c.tot1k, &D.dkp));
    RET(st.io(D.dkw, c.tot1k, &D.dkw));
    {
        long tl[12] = {c.totki, c.totki, c.tot2_l1, c.tot2_l1, c.totjk, c.totjk, c.tot2_l1, c.tot2_l1,
                       c.totjk, c.totjk, c.totki, c.totki};
        // tot2_l1 is known once the tables exist
        if (!c.d_offki) {
            long l1 = 0;
            for (int b = 1; b <= c.g.numbl; b++) l1 += (long)c.lv[1].n[b][0] * c.lv[1].n[b][1];
            for (int q : {2, 3, 6, 7}) tl[q] = l1;
        }
        for (int q = 0; q < 12; q++) {
            if (!D.tw[q]) return set_err(LES_ERR_ARG, "wall array %d missing", q);
            RET(st.io(D.tw[q], tl[q], &D.tw[q]));
        }
    }
    double *const *m = D.metric;
    double **tw = D.tw;
    const lester_ctrl &k = c.c;
    const int one = 1, iU = 1, iV = 2, iW = 3;
    double zero = 0.0;
    const double *mx[12] = {m[M_DIP], m[M_DIU], m[M_DIX], m[M_DJP], m[M_DJV], m[M_DJX],
                            m[M_RDIV], m[M_RDJU], m[M_DIDJP], m[M_RP], m[M_RU], m[M_RV]};
    // conv_exitbc(task, iva) of step.F:344 and 435
    auto exitbc = [&](int task, int iva) {
        return exit_task(c, task, iva, D.rho, D.rhonp1, D.u, D.v, D.w, D.u_int, D.v_int, D.w_int, D.hn_u, D.hn_v,
                         D.hn_w, mx, D.dkp, D.dkw, m[M_RDIDJP]);
    };
    // ---- ivar = u: the inlet planes (step.F:226)
    if (has_inlet(c))
        RET(inlet_task(c, c.d_uprof, c.d_vprof, c.inlet_seed, *istep, D.u, D.v, D.w, D.sc1, D.rho, D.u_int,
                       D.v_int, D.w_int));
    // ---- ivar = u: boundary ghosts, eddy viscosity, scalar, u predictor
    for (int iv = 1; iv <= 3; iv++) {
        double *fld = iv == 1 ? D.u : iv == 2 ? D.v : D.w;
        RET(lester_set_virt_bc(&iv, &one, fld, nullptr, D.rho, D.gam, D.vd_damping, nullptr, &zero, tw[0], tw[1],
                               tw[2], tw[3], tw[4], tw[5], tw[6], tw[7], tw[8], tw[9], tw[10], tw[11], m[M_DIP],
                               m[M_DIU], m[M_DIV], m[M_DIX], m[M_DJP], m[M_DJU], m[M_DJV], m[M_DJX], m[M_RU],
                               m[M_RV], D.dkp, D.dkw));
    }
    RET(lester_subgrid(D.gam, D.gamsc1, D.u, D.v, D.w, D.sc1, D.rho, D.sc1var, D.sc1dis, D.vd_damping, m[M_DIP],
                       m[M_DIU], m[M_DJP], m[M_DJV], D.dkp, D.dkw, m[M_HIJP], m[M_HJIP], m[M_HKIP], m[M_HKJP],
                       m[M_RP], nullptr, nullptr));
    RET(lester_set_gamsc1_bc(D.sc1, D.gamsc1, D.gamlam, m[M_DIU], m[M_DJV], D.dkp, m[M_RP]));
    RET(lester_set_sc1(D.u, D.v, D.w, D.p, D.sc1, D.rho, D.gamsc1, D.gamlam, D.hn_sc1, m[M_DIP], m[M_DIU],
                       m[M_RDIV], m[M_DJP], m[M_DJV], m[M_RDJU], m[M_DIDJP], m[M_RDIDJP], m[M_HKIP], m[M_HKJP],
                       m[M_HKIU], m[M_HKJV], m[M_RP], D.dkp, D.dkw, nullptr, nullptr));
    RET(lester_set_sc1_bc(D.sc1));
    RET(lester_set_sc1var(D.u, D.v, D.w, D.sc1, D.rho, D.sc1var, D.sc1dis, m[M_DIP], m[M_DJP], D.dkp, D.dkw,
                          m[M_RP], nullptr, nullptr));
    RET(lester_search_lib(D.sc1, D.sc1var, D.rhonp1, D.temperature, nullptr, nullptr, istep, &k.alpha, D.rho,
                          &k.rholo, &k.rhohi));
    RET(lester_set_sc1_bc(D.sc1));
    RET(lester_set_sc1_bc(D.rhonp1));
    RET(lester_set_sc1_bc(D.temperature));
    RET(lester_set_uv_int(&iU, D.u, D.v, D.w, D.p, D.rho, D.rhonp1, D.gam, D.u_int, D.hn_u, m[M_DIP], m[M_DIU],
                          m[M_DIX], m[M_RDIX], m[M_DJP], m[M_DJU], m[M_DJV], m[M_DJX], m[M_RDJP], m[M_RDJU],
                          m[M_DIDJP], m[M_DIDJU], m[M_RDIDJU], m[M_HIJP], m[M_HIJU], m[M_HJIU], m[M_HKIU],
                          m[M_HKJU], m[M_RP], m[M_RU], D.dkp, D.dkw, tw[0], tw[1], tw[2], tw[3], nullptr,
                          nullptr));
    RET(exitbc(1, 1));
    // ---- ivar = v (step.F:319-326: the v arrays in the u roles)
    RET(lester_set_uv_int(&iV, D.v, D.u, D.w, D.p, D.rho, D.rhonp1, D.gam, D.v_int, D.hn_v, m[M_DJP], m[M_DJV],
                          m[M_DJX], m[M_RDJX], m[M_DIP], m[M_DIV], m[M_DIU], m[M_DIX], m[M_RDIP], m[M_RDIV],
                          m[M_DIDJP], m[M_DJDIV], m[M_RDJDIV], m[M_HJIP], m[M_HJIV], m[M_HIJV], m[M_HKJV],
                          m[M_HKIV], m[M_RP], m[M_RV], D.dkp, D.dkw, tw[4], tw[5], tw[6], tw[7], nullptr,
                          nullptr));
    RET(exitbc(1, 2));
    // ---- ivar = w
    RET(lester_set_w_int(D.u, D.v, D.w, D.p, D.rho, D.rhonp1, D.gam, D.w_int, D.hn_w, m[M_DIP], m[M_DIU],
                         m[M_RDIV], m[M_DJP], m[M_DJV], m[M_RDJU], m[M_DIDJP], m[M_RDIDJP], m[M_HKIP], m[M_HKJP],
                         m[M_HKIU], m[M_HKJV], m[M_RP], m[M_RU], D.dkp, D.dkw, tw[10], tw[11], tw[8], tw[9],
                         nullptr, nullptr));
    RET(exitbc(1, 3));
    // ---- ivar = p
    if (*istep == 1)
        RET(lester_coeff_p(m[M_DIU], m[M_DJV], m[M_RDIV], m[M_RDJU], m[M_DIDJP], m[M_RP], D.dkp, D.dkw, D.ap, D.aw,
                           D.ae, D.as, D.an, D.al, D.ar));
    RET(lester_sour_p(m[M_DIU], m[M_DJV], m[M_RDIV], m[M_RDJU], m[M_DIDJP], D.dkp, m[M_RDIDJP], D.dkw, D.u_int,
                      D.v_int, D.w_int, D.rho, D.rhonp1, D.drhonp1dt, D.s, D.srhot, D.srhoux, nullptr, nullptr));
    c.want_norms = false;
    int rs = lester_lmg_solve(D.ap, D.aw, D.ae, D.as, D.an, D.al, D.ar, D.p, D.s, D.res, nullptr, nullptr);
    c.want_norms = true;
    // the reference carries on after nummgits cycles whatever the residual;
    // a fast solver that stops short reports it and the step continues
    if (rs && rs != LES_ERR_NOT_CONVERGED) return rs;
    RET(lester_extrap_p(D.p, nullptr, nullptr));
    RET(lester_p_ref_subtract(D.p));
    RET(lester_uvw_adv(&iU, m[M_DIU], m[M_RP], D.dkw, D.u, D.u_int, D.rhonp1, D.p, nullptr, nullptr, istep));
    RET(lester_uvw_adv(&iV, m[M_DJV], m[M_RP], D.dkw, D.v, D.v_int, D.rhonp1, D.p, nullptr, nullptr, istep));
    RET(lester_uvw_adv(&iW, m[M_DIU], m[M_RP], D.dkw, D.w, D.w_int, D.rhonp1, D.p, nullptr, nullptr, istep));
    RET(lester_slipbc(nullptr, nullptr, nullptr, m[M_DIP], m[M_DIU], m[M_DJP], m[M_DJV], D.dkp, D.u, D.v, D.v_int,
                      D.w, D.sc1, D.rho, D.p, istep));
    for (int iva = 1; iva <= 3; iva++) RET(exitbc(2, iva));
    RET(lester_swap_rhos(D.rho, D.rhonp1, D.rhonm1));
    c.iststep += 1;  // code/step.F:181, ready for the next step
    r = st.finish();
    if (r) return r;
    return rs;
}

} // extern "C"
