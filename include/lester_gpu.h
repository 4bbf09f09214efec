/*
 * lester_gpu.h -- C ABI of the GB300 implementation of the LESter
 * per-time-step hot path.
 *
 * Every routine that the reference's time-step driver (code/step.F) calls on
 * the hot path has an entry point here with the reference's routine name
 * prefixed by `lester_`, the same argument order and the same by-reference
 * calling convention (scalars as pointers, arrays as FP64 arena slices in
 * Fortran order), so a Fortran build binds them with
 *     interface; subroutine ... bind(C, name="lester_<routine>") ...
 * and keeps its own subroutine names.
 *
 * What the reference keeps in COMMON blocks (block sizes and links, boundary
 * types, time step, model and multigrid controls) is passed once to
 * lester_gpu_init / lester_gpu_set_ctrl.
 *
 * Pointers.  Every array argument may be a host pointer or a device pointer
 * (cudaMalloc / torch).  Host arrays are copied in and the outputs copied
 * back before the call returns ("strict drop-in" mode).  Device arrays are
 * used in place and the work is queued on the library's stream
 * (lester_gpu_get_stream); call lester_gpu_sync() before reading them on the
 * host.  Workspace arguments of the reference (work, offwork, ia, ra, gia,
 * gja, swap_geo, pnti) are accepted and ignored: the library owns its
 * device workspace.
 *
 * Errors.  Every entry point returns 0 on success or a negative LES_ERR_*
 * code; lester_gpu_last_error() gives a message.  No exception crosses the
 * ABI.  The reference `stop`s on the same conditions (e.g. code/solvers.F:35,
 * code/set_offset.F:149-151, code/set_interfaces.F:416-422).
 */
#ifndef LESTER_GPU_H
#define LESTER_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define LES_MAXBL 64  /* code/dim.inc:68 maxbl */
#define LES_MAXMGL 16 /* level cap; code/dim.inc:65 has maxmgl = 3 */

#define LES_OK 0
#define LES_ERR_NOT_INIT -1
#define LES_ERR_GEOM -2       /* bad block sizes, links or level request */
#define LES_ERR_ARG -3        /* bad scalar argument */
#define LES_ERR_CUDA -4       /* CUDA runtime error */
#define LES_ERR_NOMEM -5      /* device allocation failed */
#define LES_ERR_NONFINITE -6  /* NaN/Inf seen in a norm */
#define LES_ERR_NOT_CONVERGED -7
#define LES_ERR_STRUCTURE -8  /* coefficients lack the aw(i+1) = ae(i) pairing */
#define LES_ERR_TIMEOUT -9    /* a bounded device wait gave up */
#define LES_ERR_SIZE -10      /* request exceeds a stated maximum */

/* boundary-condition types, code/bc_type.inc:17-27 */
#define LES_BCT_WALL 1
#define LES_BCT_ZERO_GRAD 2
#define LES_BCT_CONVECTIVE 3
#define LES_BCT_FIXED 4
#define LES_BCT_TRACTION 6
#define LES_BCT_PERIODIC 12
#define LES_BCT_INTERFACE 13

/* solution variables, code/les.inc:102-106 */
#define LES_SV_U 1
#define LES_SV_V 2
#define LES_SV_W 3
#define LES_SV_P 4
#define LES_SV_SC1 5

/* pressure-solver algorithm (lester_ctrl.psolve) */
#define LES_PSOLVE_REFERENCE 0 /* lmg_solve exactly: lexicographic SOR order */
#define LES_PSOLVE_FP64 1      /* red-black SOR V-cycles, all FP64 */
#define LES_PSOLVE_MIXED 2     /* FP32 red-black V-cycles inside FP64 defect correction */

/* Block layout, the content of block.dat and the cb.lgrid.inc tables.
 * Blocks are 1-based in bl2bl; 0 = no neighbour. */
typedef struct lester_geom {
    int numbl;
    int maxmgl;  /* level cap for the level search (reference: 3) */
    int nummgl;  /* levels to use; 0 = as many as found */
    int gotrad;  /* 1 = polar grid (cb.gridp.inc gotrad) */
    int bl_nijkp1[LES_MAXBL][3]; /* points per axis incl. one ghost per side */
    int bl_bc[LES_MAXBL][6];     /* boundary type per side W,E,S,N,L,R */
    int bl2bl[LES_MAXBL][6];
    int bl2side[LES_MAXBL][6];
} lester_geom;

/* Controls the reference reads from COMMON (cb.control.inc, defaults.F). */
typedef struct lester_ctrl {
    double dtime;      /* time step */
    double visc;       /* molecular viscosity */
    double csles;      /* Smagorinsky / WALE constant */
    double rholo, rhohi;
    double alpha;      /* density relaxation factor exp(-dt/t_relax) */
    double ylaminar;   /* const.inc: 11.3 */
    double kappa;      /* ck: von Karman constant */
    double cwfun;      /* ca: log-law intercept term */
    double aplus;      /* van Driest A+ */
    int model;         /* 0 none, 1 Smagorinsky, 2 WALE, 3 Sigma (edge/subgrid_sigma.F) */
    /* multigrid, code/defaults.F:59-71 */
    int nummgits, numpre, numpost, numcits, meth_cycle;
    double tolf, relax_pmg, relax_pmgc;
    /* GPU solver selection */
    int psolve;        /* LES_PSOLVE_* */
    double rtol;       /* fast solvers stop at ||b-Ap||/||b|| <= rtol; with no
                          Dirichlet side (singular matrix) b is taken minus its
                          interior mean, the only part any p can match */
    int max_outer;     /* fast solvers: maximum V-cycles */
    int rb_sweeps;     /* fast solvers: red-black sweeps per smoothing step */
    int rb_coarse;     /* fast solvers: sweeps on the coarsest level (at
                          least 4 per point of its largest extent) */
    double rb_omega;   /* fast solvers: SOR factor */
    int exact;         /* FP64 physics kernels (predictor, eddy viscosity,
                          scalar): 1 = the reference's operation order, no
                          FMA, bitwise reproducible; 0 = fast build
                          (reciprocal metric tables, FMA, sqrt-based WALE
                          powers), a few units in the last place apart */
    int rb_matfree;    /* FP32 solver: 1 = form the couplings from their
                          separable (i,j) x k factors instead of reading the
                          coefficient arrays, when every coefficient matches
                          them to 1e-5 of ap; 0 = always read the arrays */
    int mg_tail;       /* fast solvers: levels with at most this many
                          interior points (all blocks) run as one single-CTA
                          launch per V-cycle; 0 = one launch per operation */
    int krylov;        /* fast solvers' outer loop: 0 = defect correction
                          p += V(b - A p); 1 = flexible conjugate gradients
                          with the V-cycle as preconditioner (FP64 vectors
                          and sums; converges where the plain cycle's
                          coarse-grid correction overshoots, e.g. on
                          strongly stretched grids); 2 = defect correction
                          until a cycle fails to halve the residual, then
                          flexible CG from the current p */
    int rb_line;       /* fast solvers: 1 = y-line zebra relaxation (a
                          tridiagonal solve along j per (i, k) column,
                          checkerboard in i + k) instead of point red-black
                          on the levels above the single-CTA tail; for
                          cells much thinner in y than in x and z */
    int autotune;      /* fast solvers: n >= 1 = the n-th solve of each
                          precision times candidate settings (red-black CTA
                          size, sweeps and omega, point or y-line smoothing,
                          tail threshold) on its own system and keeps the
                          fastest for the rest of the run
                          (lester_gpu_tuned); 0 = the controls as given */
    int phys32;        /* 1 = the predictors, scalar transport and eddy
                          viscosity compute in FP32 on the FP64 fields (the
                          les_f32 build; with exact = 1 lester_gpu_init and
                          lester_gpu_set_ctrl refuse it): the mixed path's
                          physics, its error against the FP64 path stated
                          per field by the tests */
    int step_graph;    /* 1 = lester_step replays the whole step as one CUDA
                          graph, the fast solve's cycle loop a device-side
                          conditional (WHILE) node; captured once per field
                          set and controls (istep > 1, fast psolve, device
                          or pinned host fields, autotuning finished);
                          otherwise the step runs as launched */
    int sc1_sweep;     /* in-place scalar sweep of set_sc1: 0 = automatic
                          (the tile pipeline with FP32 physics where its
                          shared-memory ring fits, else the hyperplane
                          sweep); 1 = hyperplane sweep, one cooperative
                          launch with a grid barrier per i+j+k plane; 2 =
                          tile pipeline, one CTA per (block, k, row range)
                          tile walking the planes i+j, the layers a
                          wavefront apart; 3 = one launch per i+j+k plane.
                          The exact build gives the same result bit for bit
                          with each; the builds with FMA agree to rounding. */
    int wait_limit;    /* bounded device waits (grid barrier, progress
                          flags): polls before a wait gives up and the call
                          returns LES_ERR_TIMEOUT; 0 = the default (2^24) */
    int p_guess;       /* initial pressure of lester_step's fast solves:
                          0 (default) = p(n), as the reference's lmg_solve
                          starts; 1 = linear extrapolation in time,
                          2 p(n) - p(n-1), from the second solved step on.
                          The fast solvers iterate to rtol either way (on
                          the mixing layer the extrapolated start took 8.15
                          V-cycles a step against 8.0). */
    int rb_tile;       /* 1: the FP32 solver's point red-black sweeps on a
                          one-block level run as one launch per sweep through
                          shared-memory tiles (both colours, a recomputed
                          halo); 0 (default): one launch per colour, which
                          measured faster on GB300 */
} lester_ctrl;

/* Arena slice lengths (elements) implied by the geometry. */
typedef struct lester_sizes {
    int nummgl;
    long n3_sg;  /* one 3-D field, level 1 (sg_off layout) */
    long n3_mg;  /* one 3-D field, all levels (mg_off layout) */
    long n2;     /* one 2-D metric, all levels */
    long n1k;    /* one 1-D k metric, all levels */
    long nxy;    /* one x or y vertex array, all levels */
    long nz;     /* z vertex array, all levels */
    long n2_ki;  /* one 2-D (k,i) wall array, level 1 */
    long n2_jk;  /* one 2-D (j,k) wall array, level 1 */
} lester_sizes;

/* Every field of one time step, as the reference keeps them in its arena
 * (code/step.F arguments).  3-D fields are level-1 (sg layout, n3_sg)
 * except p, s, res and the seven coefficients, which span every multigrid
 * level (n3_mg).  metric[] holds the 35 comp_metric arrays in its argument
 * order.  tw[] holds the wall-stress arrays tw_sfi, tw_nfi, tw_lfi, tw_rfi,
 * tw_wfj, tw_efj, tw_lfj, tw_rfj, tw_wfk, tw_efk, tw_sfk, tw_nfk.  Scratch
 * fields (u_int, v_int, w_int, drhonp1dt, srhot, srhoux) may be NULL. */
typedef struct lester_fields {
    double *u, *v, *w, *sc1, *rho, *rhonp1, *rhonm1, *u_int, *v_int, *w_int;
    double *hn_u, *hn_v, *hn_w, *hn_sc1, *gam, *gamsc1, *gamlam, *sc1var, *sc1dis;
    double *vd_damping, *temperature, *drhonp1dt, *srhot, *srhoux;
    double *p, *s, *res, *ap, *aw, *ae, *as, *an, *al, *ar;
    double *metric[35];
    double *dkp, *dkw;
    double *tw[12];
} lester_fields;

/* ---- lifecycle -------------------------------------------------------- */
/* Replaces the setup half of step.F:114-120 (set_offset, set_interfaces,
 * set_loop_bound tables).  No reference counterpart of its own. */
int lester_gpu_init(const lester_geom *g, const lester_ctrl *c);
int lester_gpu_set_ctrl(const lester_ctrl *c);
int lester_gpu_finalize(void);
int lester_gpu_sizes(lester_sizes *out);
int lester_gpu_block_info(int ilev, int iblk, int *nijkp1, long *offs);
int lester_gpu_sync(void);
void *lester_gpu_get_stream(void);
int lester_gpu_set_stream(void *stream);
const char *lester_gpu_last_error(void);
/* smoother rotation counter, SAVEd in code/sporlx.F:58 */
int lester_gpu_set_jumble(int jumble);
int lester_gpu_get_jumble(void);
/* launches of this library's kernels since the library was loaded */
long lester_gpu_launch_count(void);
/* statistics of the last lester_solvers / lester_lmg_solve call:
 * out[0..3] = rnorm, fnorm, enorm, vnorm of level 1 (code/norms.F:393-398),
 * out[4] = V-cycles, out[5] = ||b - A p|| / ||b|| */
int lester_gpu_solve_stats(double *out);
/* device milliseconds of the last fast solve (LES_PSOLVE_FP64 / MIXED), from
 * its first residual to its last, by CUDA events on the library stream */
int lester_gpu_solve_time(double *ms);
/* the settings the autotuner chose for precision prec (64 FP64, 32 mixed):
 * red-black threads per CTA, sweeps, omega, tail threshold and whether
 * y-line relaxation won; *done = 0 while it has not run */
int lester_gpu_tuned(int prec, int *done, int *threads, int *sweeps, double *omega, int *tail, int *line);
/* kernel timing inside a timed region: CUDA events around each launch of
 * the timed kernels -- LES_PROF_RB: the level-1 red-black smoother of the
 * fast solvers; LES_PROF_SWEEP: the in-place scalar sweep of set_sc1.
 * prof(1) clears and starts, prof(0) stops; prof_kernel returns one
 * kernel's summed milliseconds and number of timed launches; prof_read is
 * prof_kernel(LES_PROF_RB). */
#define LES_PROF_RB 0
#define LES_PROF_SWEEP 1
int lester_gpu_prof(int enable);
/* levels (bit l for level l) the fast solvers' last V-cycle smoothed with
 * one shared-memory red-black sweep per launch (k_rb_tile) instead of one
 * launch per colour; LES_PROF_RB then times those launches */
int lester_gpu_rb_tiles(int *level_mask);
int lester_gpu_prof_kernel(int which, double *ms_total, long *launches);
int lester_gpu_prof_read(double *ms_total, long *launches);
/* bytes copied host->device and device->host by calls with host arrays */
int lester_gpu_xfer_bytes(long *h2d, long *d2h);
/* forms the fast solvers took for the current coefficients: bit 0 the FP32
 * solver's couplings from separable factors (no coefficient arrays); bit 1
 * the mixed solver's double-float residual from separable double-float
 * factors, bit 2 its diagonal as their sum; bit 3 / bit 4 the bottom level
 * solved exactly by the FP32 / FP64 solver */
int lester_gpu_solver_forms(int *flags);

/* One time step: the ivar loop of code/step.F:214-454 (fixed_inlet on the
 * inlet blocks of lester_gpu_set_inlet, set_virt_bc x3, subgrid, scalar
 * transport and density, momentum predictor with conv_exitbc task 1 after
 * each component, coeff_p at istep 1, sour_p, solvers, extrap_p,
 * p_ref_subtract, uvw_adv x3, slipbc, conv_exitbc task 2, swap_rhos).
 * Host arrays: the fields a step reads, or writes only in part (u v w sc1
 * rho hn_* gam gamsc1 sc1var sc1dis vd_damping temperature, level 1 of p,
 * metrics, dkp, dkw, the wall arrays), are copied in once per call; the
 * fields the caller reads after the step (those, rhonp1, rhonm1 and gamlam,
 * without the metrics) are copied back once.  The copies run on two copy
 * streams beside the step's kernels: each input is waited for just before
 * the first routine that touches it, each output is copied back once the
 * step has finished writing it.  After an error return the host arrays
 * may hold a partly updated state.  The work arrays (u_int v_int
 * w_int drhonp1dt srhot srhoux s res, p below level 1) are library-held
 * device arrays when host arrays are passed and are not written back.  The
 * pressure coefficients, which coeff_p writes at istep 1 and no later step
 * changes, are written back at istep 1 and kept on the device for the host
 * arrays passed then; a later call with other host coefficient arrays
 * copies those in once.
 * Returns LES_ERR_NOT_CONVERGED (after completing the step) if a fast
 * pressure solver stopped at max_outer above rtol. */
int lester_step(lester_fields *fields, const int *istep);
/* No counterpart in the reference (its step.F prints wall times only): with
 * a path, every later lester_step appends one JSON line to that file --
 * istep, return code, host wall ms of the call, V-cycles, relative
 * residual, the RMS residual and right-hand side of the pressure equation
 * (code/norms.F rnorm, fnorm; the projected velocity's discrete divergence
 * is that residual), whether the step was replayed from the whole-step
 * graph, bytes copied each way.  NULL or "" closes the log. */
int lester_gpu_step_log(const char *path);

/* ---- halo exchange ---------------------------------------------------- */
/* code/swap_sc0.F:6 swap_sc(ivar1, igrid, var, work, mg_or_sg) */
int lester_swap_sc(const int *ivar1, const int *igrid, double *var,
                   double *work, const int *mg_or_sg);

/* ---- metrics ---------------------------------------------------------- */
/* code/comp_metric.F:5 comp_metric(x, y, t, dip ... rdjdiv, dkp, dkw,
 * swap_geo, pnti) */
int lester_comp_metric(const double *x, const double *y, const double *t,
                       double *dip, double *diu, double *div, double *dix,
                       double *rdip, double *rdiv, double *rdix, double *djp,
                       double *dju, double *djv, double *djx, double *rdjp,
                       double *rdju, double *rdjx, double *hijp, double *hjip,
                       double *hkip, double *hkjp, double *hiju, double *hjiu,
                       double *hkiu, double *hkju, double *hijv, double *hjiv,
                       double *hkiv, double *hkjv, double *rp, double *ru,
                       double *rv, double *didjp, double *rdidjp,
                       double *didju, double *rdidju, double *djdiv,
                       double *rdjdiv, double *dkp, double *dkw,
                       double *swap_geo, int *pnti);

/* ---- pressure path ---------------------------------------------------- */
/* code/coeff_p.F:5 coeff_p(diu, djv, rdiv, rdju, didjp, rp, dkp, dkw,
 * ap, aw, ae, as, an, al, ar) */
int lester_coeff_p(const double *diu, const double *djv, const double *rdiv,
                   const double *rdju, const double *didjp, const double *rp,
                   const double *dkp, const double *dkw, double *ap,
                   double *aw, double *ae, double *as, double *an,
                   double *al, double *ar);
/* code/sour_p.F:6 sour_p(diu, djv, rdiv, rdju, didjp, dkp, rdidjp, dkw,
 * u, v, w, rho, rhonp1, Drhonp1Dt, s, srhot, srhoux, gia, gja) */
int lester_sour_p(const double *diu, const double *djv, const double *rdiv,
                  const double *rdju, const double *didjp, const double *dkp,
                  const double *rdidjp, const double *dkw, const double *u,
                  const double *v, const double *w, const double *rho,
                  const double *rhonp1, double *drhonp1dt, double *s,
                  double *srhot, double *srhoux, double *gia, double *gja);
/* code/solvers.F:5 solvers(ap, aw, ae, as, an, al, ar, f, b, residu, ia, ra)
 * -> lmg_solve (code/lmg_solve.F:5) for psolver 101.  The algorithm follows
 * lester_ctrl.psolve.  Coarse-level parts of b and residu are overwritten,
 * as in the reference. */
int lester_solvers(const double *ap, const double *aw, const double *ae,
                   const double *as, const double *an, const double *al,
                   const double *ar, double *f, double *b, double *residu,
                   int *ia, double *ra);
int lester_lmg_solve(const double *ap, const double *aw, const double *ae,
                     const double *as, const double *an, const double *al,
                     const double *ar, double *f, double *b, double *residu,
                     int *ia, double *ra);
/* code/norms.F:5 norms(ilev, mg_or_sg, ap..ar, x, b, residu,
 * res_norm, rhs_norm, err_norm, var_norm) */
int lester_norms(const int *ilev, const int *mg_or_sg, const double *ap,
                 const double *aw, const double *ae, const double *as,
                 const double *an, const double *al, const double *ar,
                 const double *x, const double *b, double *residu,
                 double *res_norm, double *rhs_norm, double *err_norm,
                 double *var_norm);
/* No counterpart in the reference.  lester_norms for one block, for hosts
 * that must not allocate device memory when they call it (a code that runs
 * under a fixed device-memory budget, or owns all device memory through
 * its own pool and forbids libraries to allocate): it needs no
 * lester_gpu_init and allocates nothing.  Its scratch is a static device
 * array of 4 * LES_NOALLOC_MAX_POINTS / 256 + 8 doubles (512 KB); blocks
 * with more than LES_NOALLOC_MAX_POINTS interior points are rejected with
 * LES_ERR_SIZE.  nijkp1 = points per axis incl. ghosts; every array is
 * device memory of the current device, in the reference's Fortran order;
 * the call queues its work on `stream` (a cudaStream_t, NULL for the
 * default stream), waits for it and writes the norms to host scalars.
 * Nothing in the scratch has to start at zero.  Calls that overlap on the
 * GPU race on the one scratch.  The first call in each CUDA context of a
 * device (again after a cudaDeviceReset) looks up the scratch address
 * (cudaGetSymbolAddress) and should come before any stream capture. */
#define LES_NOALLOC_MAX_POINTS 4194304L
int lester_norms_noalloc(const int *nijkp1, const double *ap, const double *aw,
                         const double *ae, const double *as, const double *an,
                         const double *al, const double *ar, const double *x,
                         const double *b, double *residu, double *res_norm,
                         double *rhs_norm, double *err_norm, double *var_norm,
                         void *stream);
/* code/restriction.F:5 restriction(ilev, f, f1, work, offwork) */
int lester_restriction(const int *ilev, const double *f, double *f1,
                       double *work, int *offwork);
/* code/prolongation.F:5 prolongation(ilev, f, work, offwork) */
int lester_prolongation(const int *ilev, double *f, double *work,
                        int *offwork);
/* code/sporlx.F:5 sporlx(ilev, ap..ar, f, b, residu, niter, omega, soltol,
 * work, offwork, res_norm, rhs_norm, err_norm, var_norm) */
int lester_sporlx(const int *ilev, const double *ap, const double *aw,
                  const double *ae, const double *as, const double *an,
                  const double *al, const double *ar, double *f,
                  const double *b, double *residu, const int *niter,
                  const double *omega, const double *soltol, double *work,
                  int *offwork, double *res_norm, double *rhs_norm,
                  double *err_norm, double *var_norm);
/* code/extrap_p.F:5 extrap_p(p, work, offwork) */
int lester_extrap_p(double *p, double *work, int *offwork);
/* code/p_ref_subtract.F:6 p_ref_subtract(p) */
int lester_p_ref_subtract(double *p);
/* code/uvw_adv.F:5 uvw_adv(ivar1, diu, rp, dkw, u, u_int, rho, p, wk,
 * offwork, step) */
int lester_uvw_adv(const int *ivar1, const double *diu, const double *rp,
                   const double *dkw, double *u, const double *u_int,
                   const double *rho, const double *p, double *wk,
                   int *offwork, const int *step);
/* code/swap_rhos.F:5 swap_rhos(rho, rhonp1, rhonm1) */
int lester_swap_rhos(double *rho, double *rhonp1, double *rhonm1);
/* code/search_lib.F:5 search_lib(sc1, sc1var, rhonp1, Temperature, work,
 * offwork, istep, alpha, rho, rholo, rhohi) */
int lester_search_lib(double *sc1, double *sc1var, double *rhonp1,
                      double *temperature, double *work, int *offwork,
                      const int *istep, const double *alpha,
                      const double *rho, const double *rholo,
                      const double *rhohi);
/* code/slipbc.F:3 slipbc(x, y, z, dip, diu, djp, djv, dkp, u, v, v_int, w,
 * sc1, rho, p, step) */
int lester_slipbc(const double *x, const double *y, const double *z,
                  const double *dip, const double *diu, const double *djp,
                  const double *djv, const double *dkp, double *u, double *v,
                  const double *v_int, double *w, double *sc1, double *rho,
                  const double *p, const int *step);

/* ---- momentum predictor ----------------------------------------------- */
/* the step counter iststep of code/step.F:167,181 (wall-stress running
 * means): the value the next predictor call and the next lester_step use.
 * It starts at 2, the value of a run's first step; lester_step advances it
 * by one after each step. */
int lester_gpu_set_iststep(int iststep);
/* No counterpart in the reference: a body force per unit volume for the u,
 * v and w predictors (device arrays in the level-1 layout, NULL = none),
 * added to each component's explicit term h.  It is the control of the
 * adjoint (lester_adjoint_run); the reference has no forcing term. */
int lester_gpu_set_body_force(const double *fu, const double *fv, const double *fw);
/* code/set_uv_int.F:5 set_uv_int(iva, u, v, w, p, rho, rhonp1, gam, u_int,
 * hu, dip, diu, dix, rdix, djp, dju, djv, djx, rdjp, rdju, didjp, didju,
 * rdidju, hijp, hiju, hjiu, hkiu, hkju, rp, ru, dkp, dkw, tw_sfi, tw_nfi,
 * tw_lfi, tw_rfi, work, offwork).  For iva = 2 the caller passes the v
 * arrays in the u roles, as code/step.F:319-326 does. */
int lester_set_uv_int(const int *iva, const double *u, const double *v,
                      const double *w, const double *p, const double *rho,
                      const double *rhonp1, const double *gam, double *u_int,
                      double *hu, const double *dip, const double *diu,
                      const double *dix, const double *rdix, const double *djp,
                      const double *dju, const double *djv, const double *djx,
                      const double *rdjp, const double *rdju,
                      const double *didjp, const double *didju,
                      const double *rdidju, const double *hijp,
                      const double *hiju, const double *hjiu,
                      const double *hkiu, const double *hkju, const double *rp,
                      const double *ru, const double *dkp, const double *dkw,
                      double *tw_sfi, double *tw_nfi, double *tw_lfi,
                      double *tw_rfi, double *work, int *offwork);
/* code/set_w_int.F:5 set_w_int(u, v, w, p, rho, rhonp1, gam, w_int, hw, dip,
 * diu, rdiv, djp, djv, rdju, didjp, rdidjp, hkip, hkjp, hkiu, hkjv, rp, ru,
 * dkp, dkw, tw_sfk, tw_nfk, tw_wfk, tw_efk, work, offwork) */
int lester_set_w_int(const double *u, const double *v, const double *w,
                     const double *p, const double *rho, const double *rhonp1,
                     const double *gam, double *w_int, double *hw,
                     const double *dip, const double *diu, const double *rdiv,
                     const double *djp, const double *djv, const double *rdju,
                     const double *didjp, const double *rdidjp,
                     const double *hkip, const double *hkjp, const double *hkiu,
                     const double *hkjv, const double *rp, const double *ru,
                     const double *dkp, const double *dkw, double *tw_sfk,
                     double *tw_nfk, double *tw_wfk, double *tw_efk,
                     double *work, int *offwork);

/* code/set_virt_bc.F:8 set_virt_bc(iva, ilev, f, fm, rho, gam, vd_damping,
 * init_vdd, value, tw_sfi, tw_nfi, tw_lfi, tw_rfi, tw_wfj, tw_efj, tw_lfj,
 * tw_rfj, tw_wfk, tw_efk, tw_sfk, tw_nfk, dip, diu, div, dix, djp, dju, djv,
 * djx, ru, rv, dkp, dkw) for the velocities at ilev = 1: log-law / no-slip
 * ghost values on wall sides and the van Driest damping field.  init_vdd is
 * kept by the library. */
int lester_set_virt_bc(const int *iva, const int *ilev, double *f,
                       const double *fm, const double *rho, const double *gam,
                       double *vd_damping, int *init_vdd, const double *value,
                       double *tw_sfi, double *tw_nfi, double *tw_lfi,
                       double *tw_rfi, double *tw_wfj, double *tw_efj,
                       double *tw_lfj, double *tw_rfj, double *tw_wfk,
                       double *tw_efk, double *tw_sfk, double *tw_nfk,
                       const double *dip, const double *diu, const double *div,
                       const double *dix, const double *djp, const double *dju,
                       const double *djv, const double *djx, const double *ru,
                       const double *rv, const double *dkp, const double *dkw);

/* ---- scalar transport ------------------------------------------------- */
/* code/set_gamsc1_bc.F set_gamsc1_bc(sc1, gamsc1, gamlam, diu, djv, dkp, rp) */
int lester_set_gamsc1_bc(const double *sc1, double *gamsc1, double *gamlam,
                         const double *diu, const double *djv,
                         const double *dkp, const double *rp);
/* code/set_sc1.F:5 set_sc1(u, v, w, p, sc1, rho, gamsc1, gamlam, hsc1, dip,
 * diu, rdiv, djp, djv, rdju, didjp, rdidjp, hkip, hkjp, hkiu, hkjv, rp, dkp,
 * dkw, work, offwork) */
int lester_set_sc1(const double *u, const double *v, const double *w,
                   const double *p, double *sc1, const double *rho,
                   const double *gamsc1, const double *gamlam, double *hsc1,
                   const double *dip, const double *diu, const double *rdiv,
                   const double *djp, const double *djv, const double *rdju,
                   const double *didjp, const double *rdidjp,
                   const double *hkip, const double *hkjp, const double *hkiu,
                   const double *hkjv, const double *rp, const double *dkp,
                   const double *dkw, double *work, int *offwork);
/* code/set_sc1_bc.F set_sc1_bc(sc1) */
int lester_set_sc1_bc(double *sc1);
/* code/set_sc1var.F set_sc1var(u, v, w, sc1, rho, sc1var, sc1dis, dip, djp,
 * dkp, dkw, rp, work, offwork) */
int lester_set_sc1var(const double *u, const double *v, const double *w,
                      const double *sc1, const double *rho, double *sc1var,
                      double *sc1dis, const double *dip, const double *djp,
                      const double *dkp, const double *dkw, const double *rp,
                      double *work, int *offwork);

/* ---- eddy viscosity --------------------------------------------------- */
/* code/subgrid.F:5 subgrid(gam, gamsc1, u, v, w, sc1, rho, sc1var, sc1dis,
 * vd_damping, dip, diu, djp, djv, dkp, dkw, hijp, hjip, hkip, hkjp, rp,
 * work, offwork) */
int lester_subgrid(double *gam, double *gamsc1, const double *u,
                   const double *v, const double *w, const double *sc1,
                   const double *rho, double *sc1var, double *sc1dis,
                   const double *vd_damping, const double *dip,
                   const double *diu, const double *djp, const double *djv,
                   const double *dkp, const double *dkw, const double *hijp,
                   const double *hjip, const double *hkip, const double *hkjp,
                   const double *rp, double *work, int *offwork);

/* ---- convective outflow and fixed inflow sides ------------------------ */
/* code/conv_exitbc.F:21 conv_exitbc(task, iva, rho, rhonp1, u, v, w,
 * u_int, v_int, w_int, hu, hv, hw, dip, diu, dix, djp, djv, djx, rdiv,
 * rdju, didjp, rp, ru, rv, dkp, dkw, rdidjp).  Task 1 (after the predictor
 * of variable iva, step.F:344): the exit planes of BCT_CONVECTIVE sides get
 * u_int from the convective condition with the side's mean outflow
 * velocity of step n, and at iva = 3 the exit velocities are scaled so the
 * outflow matches the inflow of the BCT_FIXED sides minus the mass change.
 * Task 2 (after the projection, step.F:433-441): the exit planes take
 * u_int.  The SAVEd values between calls live on the device.  No-op
 * without convective sides; a convective low-z side is refused
 * (LES_ERR_GEOM: the reference reads below the block there). */
int lester_conv_exitbc(const int *task, const int *iva, const double *rho, const double *rhonp1, double *u,
                       double *v, double *w, double *u_int, double *v_int, double *w_int, double *hu, double *hv,
                       double *hw, const double *dip, const double *diu, const double *dix, const double *djp,
                       const double *djv, const double *djx, const double *rdiv, const double *rdju,
                       const double *didjp, const double *rp, const double *ru, const double *rv,
                       const double *dkp, const double *dkw, const double *rdidjp);
/* code/mass_change.F:6 mass_change(rho, rhonp1, mass_chg, rdidjp, dkw):
 * sum over interior cells of (rhonp1 - rho) rdidjp dkw / dtime. */
int lester_mass_change(const double *rho, const double *rhonp1, double *mass_chg, const double *rdidjp,
                       const double *dkw);
/* The inlet configuration fixed_inlet reads from COMMON (inlet1..inlet4:
 * 1-based block numbers, 0 = none) and the profiles read_profile reads
 * from inflowbc.3d (fixed_inlet.F:187-227): nprof values of u and v, host
 * or device arrays, copied.  `seed` keys the inlet perturbations that
 * lester_step draws. */
int lester_gpu_set_inlet(const int *inlet, const double *uprof, const double *vprof, int nprof,
                         unsigned long long seed);
/* code/fixed_inlet.F:5 fixed_inlet(hu, hv, hw, u_int, v_int, w_int, u, v,
 * w, p, sc1, rho, gam, iseed, y, uprof, vprof, wprof, uuprof, vvprof,
 * wwprof, umean, vmean, wmean, uumean, vvmean, wwmean, step): the inflow
 * plane (i = 2 faces, i = 1 ghosts) of each inlet block from the profiles
 * plus a perturbation 0.005 a (2 U - 1), U uniform in [0, 1).  The
 * reference draws U with the Fortran random_number; here U is a
 * counter-based function of (iseed, step, block, j, k).  Only uprof and
 * vprof (length nprof of lester_gpu_set_inlet) are read. */
int lester_fixed_inlet(double *hu, double *hv, double *hw, double *u_int, double *v_int, double *w_int, double *u,
                       double *v, double *w, const double *p, double *sc1, double *rho, const double *gam,
                       const int *iseed, const double *y, const double *uprof, const double *vprof,
                       const double *wprof, const double *uuprof, const double *vvprof, const double *wwprof,
                       const double *umean, const double *vmean, const double *wmean, const double *uumean,
                       const double *vvmean, const double *wwmean, const int *step);

/* mas-recyc/recycling.F:5 recycling(hu, hv, hw, u_int, v_int, w_int, u, v,
 * w, p, sc1, rho, gam, iseed, y, uprof, vprof, wprof, uuprof, vvprof,
 * wwprof, umean, vmean, wmean, uumean, vvmean, wwmean, step, inblock):
 * recycling-rescaling inflow on the chain of blocks inblock..inblock+7 --
 * running plane means and rms of u, v, w per j (relaxation 0.144), every
 * 100th step from step 200 the chain rescaled to the target profiles, and
 * the plane i = 3 of block inblock+7 copied into the inflow plane of block
 * inblock (scalar 1, density rhohi).  The 1-D arrays have the length nprof
 * of lester_gpu_set_inlet; the reference's file reads and writes of the
 * running means are the caller's.  Call it immediately before lester_step,
 * the position of its call in that program's step.F. */
int lester_recycling(double *hu, double *hv, double *hw, double *u_int, double *v_int, double *w_int, double *u,
                     double *v, double *w, const double *p, double *sc1, double *rho, const double *gam, const int *iseed,
                     const double *y, const double *uprof, const double *vprof, const double *wprof,
                     const double *uuprof, const double *vvprof, const double *wwprof, double *umean, double *vmean,
                     double *wmean, double *uumean, double *vvmean, double *wwmean, const int *step,
                     const int *inblock);

/* ---- statistics ------------------------------------------------------- */
/* code/statistics.F:1 statistics(u, v, w, p, rho, um, vm, wm, pm, rhom, ruv,
 * rvw, rwu, ruu, rvv, rww, rrh, gam, gamsc1, sc1, fm, rff, sc1var, sc1dis,
 * sc1varm, sc1dism, Temperature, T_m, dip, djp, rp, dkp, dkw, x, y, z,
 * step): span (k) averages of rho u, rho v, rho w, p, rho and the second
 * moments, the scalar, its square and variance, and gam (into T_m, as the
 * reference stores it), folded into running means over no_sam samples
 * (lester_gpu_set_stat_samples; the COMMON no_sam).  The 2-D outputs use
 * the level-1 layout of the 2-D metrics.  Velocities are cell-centred as
 * statistics.F's centre does; its unset edge cells are 0 here.  The file
 * outputs are not part of this call. */
int lester_gpu_set_stat_samples(int no_sam);
int lester_statistics(const double *u, const double *v, const double *w, const double *p, const double *rho,
                      double *um, double *vm, double *wm, double *pm, double *rhom, double *ruv, double *rvw,
                      double *rwu, double *ruu, double *rvv, double *rww, double *rrh, const double *gam,
                      const double *gamsc1, const double *sc1, double *fm, double *rff, const double *sc1var,
                      const double *sc1dis, double *sc1varm, double *sc1dism, const double *temperature, double *t_m,
                      const double *dip, const double *djp, const double *rp, const double *dkp, const double *dkw,
                      const double *x, const double *y, const double *z, const int *step);

/* Steps run by replaying the whole-step graph (ctrl.step_graph) since
 * lester_gpu_init; of those, the steps whose pressure solve the host loop
 * finished (krylov 2: a defect-correction cycle failed to halve the
 * residual, so the solve continues in flexible CG; krylov 1: the CG
 * residual missed the tolerance once recomputed); 1 in *failed if the graph
 * for the current fields and controls could not be captured (those steps
 * run as launched), with the reason in why (why_len bytes, NUL-terminated;
 * may be NULL).  No counterpart in the reference. */
int lester_gpu_step_graph_info(long *replays, long *handovers, int *failed, char *why, int why_len);

/* ---- adjoint and tangent-linear runs ---------------------------------- */
/* No counterpart in the reference.  A run of nsteps lester_step calls from
 * the state in `fields` (device arrays; the caller's arrays are not
 * changed) and the objective
 *   J = mean over steps j_first..j_last (1-based) of the mean wall shear
 *       stress visc * u / (0.5 * dju) over the first interior u points of
 *       the WALL y sides (S, N),
 * differentiated with respect to the body force of lester_gpu_set_body_force
 * (per unit volume; the current one is the linearisation point).
 * lester_adjoint_run returns J and dJ/dfu, dJ/dfv, dJ/dfw (device arrays in
 * the level-1 layout, overwritten) by the transposed step, with the state
 * checkpointed every `checkpoint` steps and each segment recomputed.
 * lester_tangent_run returns J and the directional derivative dJ along
 * (dfu, dfv, dfw) by the linearised step.  Scope: psolve FP64 or MIXED
 * (converged: the linearisation of an iterative solve is the exact solve),
 * rholo == rhohi, model 0 or 1 (Smagorinsky, Cartesian, walls only on the
 * y sides), no ZERO_GRAD sides, wall points in the laminar branch of the
 * wall function (y+ below ylaminar).  Errors as lester_step; LES_ERR_ARG
 * outside that scope. */
typedef struct lester_adj_cfg {
    int nsteps;
    int j_first, j_last;  /* objective window, 1 <= j_first <= j_last <= nsteps */
    int checkpoint;       /* steps per checkpoint segment (>= 1) */
} lester_adj_cfg;
int lester_adjoint_run(const lester_adj_cfg *cfg, const lester_fields *fields, double *J, double *gfu,
                       double *gfv, double *gfw);
int lester_tangent_run(const lester_adj_cfg *cfg, const lester_fields *fields, const double *dfu,
                       const double *dfv, const double *dfw, double *J, double *dJ);

#ifdef __cplusplus
}
#endif
#endif
