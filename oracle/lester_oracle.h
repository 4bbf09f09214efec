/*
 * lester_oracle.h -- CPU parity oracle for the LESter per-time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, single-threaded, FP64
 * restatement of the reference Fortran routines (LESter, code/ directory),
 * written loop for loop from the cited sources.  It exists so that the tests,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py can check the
 * CUDA implementation.  Nothing in the product library links or calls it.
 *
 * Parity status: UNPINNED.  The reference ships no tests, fixtures or golden
 * output, and it cannot be compiled here (Fortran 77 + MPI, no Fortran
 * compiler in the image), so this restatement is checked only against
 * known-answer properties (see tests/test_oracle_kat.py) and not against the
 * reference binary itself.
 *
 * Conventions.  Arrays are the reference's arena slices: FP64, Fortran
 * (column-major, i fastest) order, 1-based index arithmetic done with the
 * A(p, idx) macro below.  Multigrid arrays hold every level, level after
 * level, block after block (mg_off).  Block numbers in bl2bl are 1-based and
 * 0 means "no neighbour", as in block.dat.  Build with -ffp-contract=off so
 * the arithmetic is the same on x86-64 and aarch64.
 */
#ifndef LESTER_ORACLE_H
#define LESTER_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAXBL 64
#define ORC_MAXMGL 16

/* boundary-condition codes (code/bc_type.inc:17-27) */
#define ORC_BCT_WALL 1
#define ORC_BCT_ZERO_GRAD 2
#define ORC_BCT_CONVECTIVE 3
#define ORC_BCT_FIXED 4
#define ORC_BCT_TRACTION 6
#define ORC_BCT_PERIODIC 12
#define ORC_BCT_INTERFACE 13

/* solution-variable codes (code/les.inc:102-106) */
#define ORC_SV_U 1
#define ORC_SV_V 2
#define ORC_SV_W 3
#define ORC_SV_P 4
#define ORC_SV_SC1 5

/* number of 2-D metric arrays produced by comp_metric, in its argument order
 * (code/comp_metric.F:5-14): dip diu div dix rdip rdiv rdix djp dju djv djx
 * rdjp rdju rdjx hijp hjip hkip hkjp hiju hjiu hkiu hkju hijv hjiv hkiv hkjv
 * rp ru rv didjp rdidjp didju rdidju djdiv rdjdiv */
#define ORC_NMETRIC 35

typedef struct orc_ctx orc_ctx;

typedef struct {
    int nummgits;     /* max V-cycles            (code/defaults.F:59-71) */
    int numpre;       /* pre-smoothing sweeps     */
    int numpost;      /* post-smoothing sweeps    */
    int numcits;      /* coarsest-grid sweeps     */
    int meth_cycle;   /* 1 = V, 2 = F             */
    int meth_smooth;  /* 1 = sporlx               */
    int meth_csolve;  /* 0 = smoother on coarsest */
    double tolf;      /* enorm/vnorm stop tolerance */
    double relax_pmg; /* SOR omega                */
    double relax_pmgc;/* SOR omega, coarsest grid */
    int compat;       /* orc_step only, not in the reference: 1 = solve for
                         the pressure source minus its interior mean over all
                         blocks (one connected component), the compatible part
                         of a singular system, as the GPU fast solvers do; 0 =
                         the source as sour_p leaves it (the reference) */
} orc_mgctrl;

/* ---- geometry ---------------------------------------------------------- */
orc_ctx *orc_create(int numbl, const int *nijkp1, const int *bc,
                    const int *bl2bl, const int *bl2side,
                    int maxmgl, int nummgl_req, int *status);
void orc_destroy(orc_ctx *c);
/* out[0]=nummgl out[1]=mg 3-D total out[2]=level-1 3-D total
 * out[3]=2-D ij total (all levels) out[4]=1-D k total out[5]=xy total
 * out[6]=z total out[7]=2-D ki total (level 1) out[8]=2-D jk total (level 1) */
void orc_sizes(const orc_ctx *c, long *out);
/* per (level, block): nijkp1[3], mult[3], off3d, off2d_ij, off1d_k, off2d_xy,
 * off1d_z, off2d_ki, off2d_jk  (levels and blocks are 1-based) */
void orc_block_info(const orc_ctx *c, int ilev, int iblk, int *nijk,
                    int *mult, long *offs);
void orc_set_loop_bound(orc_ctx *c, int ivar);
double orc_npts_all(const orc_ctx *c, int ilev);
void orc_set_jumble(orc_ctx *c, int jumble);
int orc_get_jumble(const orc_ctx *c);

/* ---- halo exchange ----------------------------------------------------- */
void orc_swap_sc(orc_ctx *c, int igrid, double *var, int mg_or_sg);

/* ---- metrics ----------------------------------------------------------- */
void orc_comp_metric(orc_ctx *c, const double *x, const double *y,
                     const double *z, double *metric, double *dkp,
                     double *dkw, int gotrad);

/* ---- pressure path ----------------------------------------------------- */
void orc_coeff_p(orc_ctx *c, const double *diu, const double *djv,
                 const double *rdiv, const double *rdju, const double *didjp,
                 const double *rp, const double *dkp, const double *dkw,
                 double *ap, double *aw, double *ae, double *as, double *an,
                 double *al, double *ar);
void orc_sour_p(orc_ctx *c, double dtime, const double *diu,
                const double *djv, const double *rdiv, const double *rdju,
                const double *didjp, const double *dkp, const double *rdidjp,
                const double *dkw, const double *u, const double *v,
                const double *w, const double *rho, const double *rhonp1,
                double *drhodt, double *s, double *srhot, double *srhoux);
void orc_norms(orc_ctx *c, int ilev, int mg_or_sg, const double *ap,
               const double *aw, const double *ae, const double *as,
               const double *an, const double *al, const double *ar,
               const double *x, const double *b, double *residu,
               double *out4);
void orc_restriction(orc_ctx *c, int ilev, const double *f, double *f1);
void orc_prolongation(orc_ctx *c, int ilev, double *f);
void orc_sporlx(orc_ctx *c, int ilev, const double *ap, const double *aw,
                const double *ae, const double *as, const double *an,
                const double *al, const double *ar, double *f,
                const double *b, double omega, double soltol, double *out4);
void orc_lmg_solve(orc_ctx *c, const orc_mgctrl *m, const double *ap,
                   const double *aw, const double *ae, const double *as,
                   const double *an, const double *al, const double *ar,
                   double *f, double *b, double *residu,
                   double *norms_out);
void orc_extrap_p(orc_ctx *c, double *p);
void orc_p_ref_subtract(orc_ctx *c, double *p);
void orc_uvw_adv(orc_ctx *c, int ivar, double dtime, const double *diu,
                 const double *rp, const double *dkw, double *u,
                 const double *u_int, const double *rho, const double *p);
void orc_swap_rhos(orc_ctx *c, double *rho, double *rhonp1, double *rhonm1);
void orc_search_lib(orc_ctx *c, double *sc1, double *rhonp1,
                    double alpha, const double *rho, double rholo,
                    double rhohi);
void orc_slipbc(orc_ctx *c, double dtime, const double *djp, double *u,
                double *v, const double *v_int, double *w, double *sc1,
                double *rho, const double *p);

/* ---- momentum predictor ------------------------------------------------ */
/* iva = 1: u.  iva = 2: v, called as step.F:319-326 does -- pass the v field
 * as `u` and the u field as `v`; tw_* are that component's wall arrays. */
void orc_set_uv_int(orc_ctx *c, int iva, double dtime, int iststep, double visc,
                    double ylaminar, double kappa, double cwfun, const double *u,
                    const double *v, const double *w, const double *p, const double *rho,
                    const double *rhonp1, const double *gam, double *u_int, double *hu,
                    const double *metric, const double *dkp, const double *dkw, double *tw_s,
                    double *tw_n, double *tw_l, double *tw_r);
void orc_set_w_int(orc_ctx *c, double dtime, int iststep, double visc, double ylaminar,
                   double kappa, double cwfun, const double *u, const double *v,
                   const double *w, const double *p, const double *rho, const double *rhonp1,
                   const double *gam, double *w_int, double *hw, const double *metric,
                   const double *dkp, const double *dkw, double *tw_sfk, double *tw_nfk,
                   double *tw_wfk, double *tw_efk);

/* ---- wall ghost velocities --------------------------------------------- */
void orc_set_virt_bc(orc_ctx *c, int iva, double visc, double kappa, double aplus,
                     double ylaminar, double *f, const double *rho, double *vdd,
                     const double *metric, const double *dkp, const double *dkw,
                     double *const *tw);

/* ---- scalar transport -------------------------------------------------- */
void orc_set_gamsc1_bc(orc_ctx *c, double visc, const double *sc1, double *gamsc1,
                       double *gamlam, const double *metric, const double *dkp);
void orc_set_sc1(orc_ctx *c, double dtime, const double *metric, const double *dkp,
                 const double *dkw, const double *u, const double *v, const double *w,
                 double *sc1, double *hsc1, const double *rho, const double *gamsc1,
                 const double *gamlam);
void orc_set_sc1_bc(orc_ctx *c, double *f);
void orc_set_sc1var(orc_ctx *c, const double *sc1, double *sc1var, const double *metric,
                    const double *dkp, const double *dkw);

/* ---- one time step ------------------------------------------------------ */
typedef struct {
    double dtime, visc, csles, rholo, rhohi, alpha, ylaminar, kappa, cwfun, aplus;
    int model, gotrad;
} orc_phys;

/* the step's fields; metric is the flat 35 x tot2 comp_metric table, tw[]
 * are tw_sfi tw_nfi tw_lfi tw_rfi tw_wfj tw_efj tw_lfj tw_rfj tw_wfk tw_efk
 * tw_sfk tw_nfk */
typedef struct {
    double *u, *v, *w, *sc1, *rho, *rhonp1, *rhonm1, *u_int, *v_int, *w_int;
    double *hn_u, *hn_v, *hn_w, *hn_sc1, *gam, *gamsc1, *gamlam, *sc1var, *sc1dis;
    double *vd_damping, *temperature, *drhonp1dt, *srhot, *srhoux;
    double *p, *s, *res, *ap, *aw, *ae, *as, *an, *al, *ar;
    double *metric, *dkp, *dkw;
    double *tw[12];
} orc_fields;

void orc_step(orc_ctx *c, const orc_mgctrl *mg, const orc_phys *k, int istep, int iststep,
              orc_fields *F);

/* ---- convective outflow and fixed inflow (orc_outflow.c) ---------------- */
int orc_has_convective(const orc_ctx *c);
/* code/conv_exitbc.F:21: task 1 after each predictor (iva = ivar), task 2
   after the projection; metric = the 35 packed 2-D metrics */
void orc_conv_exitbc(orc_ctx *c, int task, int iva, double dtime, const double *rho,
                     const double *rhonp1, double *u, double *v, double *w, double *u_int,
                     double *v_int, double *w_int, double *hu, double *hv, double *hw,
                     const double *metric, const double *dkp, const double *dkw);
/* code/mass_change.F:6: sum over cells of (rhonp1 - rho) vol / dt */
double orc_mass_change(orc_ctx *c, double dtime, const double *rho, const double *rhonp1,
                       const double *rdidjp, const double *dkw);
/* counter-based uniform [0, 1) of the inlet perturbations */
double orc_inlet_uniform(unsigned long long seed, int step, int block, int j, int k);
/* code/fixed_inlet.F:5 on the blocks inlet[0..3] (1-based, 0 = none) */
void orc_fixed_inlet(orc_ctx *c, const int inlet[4], const double *uprof, const double *vprof,
                     unsigned long long seed, int step, double rholo, double rhohi, double *u,
                     double *v, double *w, double *sc1, double *rho, double *u_int, double *v_int,
                     double *w_int);
/* mas-recyc/recycling.F:5 on blocks inblock..inblock+7 (1-based) */
void orc_recycling(orc_ctx *c, int step, int inblock, const int inlet[4], double rhohi, double *u, double *v,
                   double *w, double *sc1, double *rho, double *u_int, double *v_int, double *w_int,
                   const double *uprof, const double *vprof, const double *wprof, const double *uuprof,
                   const double *vvprof, const double *wwprof, double *umean, double *vmean, double *wmean,
                   double *uumean, double *vvmean, double *wwmean);
/* code/statistics.F:1-200: span-averaged running statistics, outs = the 2-D
   arrays um vm wm pm rhom ruv rvw rwu ruu rvv rww rrh fm rff sc1varm T_m */
void orc_statistics(orc_ctx *c, int no_sam, const double *u, const double *v, const double *w, const double *p,
                    const double *rho, const double *sc1, const double *sc1var, const double *gam,
                    double *const *outs);
/* inlet configuration used by orc_step (profiles copied, nprof values each) */
void orc_set_inlet(orc_ctx *c, const int inlet[4], const double *uprof, const double *vprof,
                   int nprof, unsigned long long seed);

/* ---- eddy viscosity ---------------------------------------------------- */
void orc_subgrid(orc_ctx *c, int model, double csles, int gotrad, double alpha,
                 double *gam, double *gamsc1, const double *u,
                 const double *v, const double *w, const double *sc1,
                 double *sc1var, double *sc1dis, const double *vd_damping,
                 const double *dip, const double *diu, const double *djp,
                 const double *djv, const double *dkp, const double *dkw,
                 const double *hijp, const double *hjip, const double *hkip,
                 const double *hkjp, const double *rp);

#ifdef __cplusplus
}
#endif
#endif
