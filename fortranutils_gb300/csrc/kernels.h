// kernels.h -- host-side launchers of the device kernels (one namespace,
// all asynchronous on the given stream).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "k_common.cuh"
#include "phys_args.h"

namespace les {

// running count of kernel launches made by this library
void count_launch(long n);
long launch_count();  // kernels launched so far (count_launch's total)

// k_exact.cu
void launch_halo(const FaceDev *faces, int nface, long maxface, double *var, double *work,
                 cudaStream_t st);
void launch_coeff_p(const BlkDev *blk, int nb, long maxcell, const double *const *m,
                    const double *dkp, const double *dkw, double *const *a, cudaStream_t st);
void launch_sour_p(const BlkDev *blk, int nb, long maxcell, double dtime, const double *rdiv,
                   const double *rdju, const double *didjp, const double *dkp,
                   const double *rdidjp, const double *dkw, const double *u, const double *v,
                   const double *w, const double *rho, const double *rhonp1, double *drhodt,
                   double *s, double *srhot, double *srhoux, cudaStream_t st);
long norms_parts(int nb, long maxcell);
void launch_norms(const BlkDev *blk, int nb, long maxcell, const double *const *a, const double *x,
                  const double *b, double *residu, double *partial, double rnpts, double *out,
                  cudaStream_t st);
void launch_lex_pass(const BlkDev *blk, int nb, int maxjk, int smin, int smax, int dir,
                     double omega, const double *const *a, double *f, const double *src,
                     double *nrm3, int want_norm, cudaStream_t st);
void launch_lex_norm(const BlkDev *blk, int nb, long maxcell, const double *nrm3, double *partial,
                     double rnpts, double *out, cudaStream_t st);
void launch_restrict(const BlkDev *bc, const BlkDev *bf, int nb, long maxcell_c, const double *ff,
                     double *fc, cudaStream_t st);
void launch_prolong(const BlkDev *bc, const BlkDev *bf, int nb, long maxfine, double *f,
                    cudaStream_t st);
void launch_extrap_p(const BlkDev *blk, int nb, double *p, cudaStream_t st);
void launch_pref(const BlkDev *blk, double *p, long n, double *scratch, cudaStream_t st);
void launch_uvw_adv(const BlkDev *blk, int nb, long maxcell, int ivar, double dtime,
                    const double *dg, const double *rp, const double *dkw, double *u,
                    const double *u_int, const double *rho, const double *p, bool f32, cudaStream_t st);
void launch_swap_rhos(double *rho, const double *rhonp1, double *rhonm1, long n, cudaStream_t st);
// double-float outer iteration of the mixed solver (k_dfloat.cu)
void launch_df_split(const double *src, float2 *dst, long n, cudaStream_t st);
void launch_df_split_b(const BlkDev *blk, int nb, long maxcell, const double *b, const double *shift, float2 *dst,
                       cudaStream_t st);
// cycles (nullable, device): skipped when *cycles == 0
void launch_df_join(const float2 *src, double *dst, long n, const double *cycles, cudaStream_t st);
void launch_df_update(const BlkDev *blk, int nb, const int maxn[3], float2 *p, const float *e, const PushDev *push,
                      bool wide, ZMap zm, cudaStream_t st);
// separable double-float factors of the level-1 FP64 couplings (E, N, R,
// P: the FP64 arrays) and their check against every interior point within
// tol * ap: bad |= 1 (couplings), 2 (diagonal not their sum), 16 (a zero
// reference coupling)
int launch_df_mf(const BlkDev *blk, int nb, long maxcell, long max2d, int maxn2, const double *E, const double *N,
                 const double *R, const double *P, const DfTab &t, double tol, int *bad, cudaStream_t st);
// the double-float residual from those factors; P NULL: the diagonal as the
// couplings' sum
void launch_df_resid_mf(const BlkDev *blk, int nb, long maxrow, const DfTab &t, const float2 *P, const float2 *x,
                        const float2 *b, float *rT, double *partial, double *out, cudaStream_t st);
void launch_df_resid(const BlkDev *blk, int nb, long maxrow, const float2 *E, const float2 *N, const float2 *R,
                     const float2 *P, const float2 *x, const float2 *b, float *rT, double *partial, double *out,
                     cudaStream_t st);
// f32: FP32 arithmetic on the FP64 fields (the mixed path with FP32 physics)
void launch_search_lib(double *sc1, double *rhonp1, const double *rho, double alpha, double rholo,
                       double rhohi, long n, bool f32, cudaStream_t st);
void launch_slipbc(const BlkDev *blk, int nb, long maxik, double dtime, const double *djp,
                   double *u, double *v, const double *v_int, double *w, double *sc1,
                   double *rho, const double *p, cudaStream_t st);

// k_metric.cu
void launch_metric(const void *metblk, int nb, long maxij, long maxk, const double *x,
                   const double *y, const double *z, double *const *m, double *dkp, double *dkw,
                   int gotrad, cudaStream_t st);
void launch_metric_swap(const void *faces, int nf, long maxlen, double *const *m, double *dkp,
                        double *dkw, double *buf, long slot, int phase, cudaStream_t st);
size_t metblk_size();
size_t metface_size();
void fill_metblk(void *dst, int idx, const int *n, long off2, long off1k, long offxy, long offz);
void fill_metface(void *dst, int idx, long src2, long dst2, long stride, long sstride, int len,
                  long srck, long dstk);


// k_fast.cu (T = float or double)
template <typename T>
int launch_conv_coef(const BlkDev *blk, int nb, long maxcell, const double *const *a, T *E, T *N,
                     T *R, T *D, double *E64, double *N64, double *R64, double *P64, int *bad,
                     cudaStream_t st);
// red-black half sweep: CTAs of `threads` (128, 256, 512) = 32 points of a
// row x 4, 8 or 16 rows; maxn: the most points of a block along i, j, k
// (ghosts included); wide: 64-bit offsets (arrays of 2^31 points or more);
// geo (nullable): the level as a kernel parameter (at most kGeoBlk blocks)
template <typename T>
void launch_rb(const BlkDev *blk, int nb, const int maxn[3], int color, double omega, const T *E,
               const T *N, const T *R, const T *D, T *x, const T *b, const PushDev *push,
               const MfTab<T> &mf, int threads, bool wide, const LevGeo *geo, ZMap zm, cudaStream_t st);
// y-line zebra relaxation of one colour of (i, k) columns (maxik_half: the
// most columns of one colour in a block)
template <typename T>
void launch_yline(const BlkDev *blk, int nb, long maxik_half, int color, double omega, const T *E, const T *N,
                  const T *R, const T *D, T *x, const T *b, const MfTab<T> &mf, T *cp, T *dp, int maxnj,
                  cudaStream_t st);
template <typename T>
void launch_resid_restrict(const BlkDev *bc, const BlkDev *bf, int nb, const int maxn_c[3], const T *E,
                           const T *N, const T *R, const T *D, const T *x, const T *b, T *bcoarse,
                           const MfTab<T> &mf, bool wide, ZMap zm_c, cudaStream_t st);
template <typename T>
void launch_vtail(const VLev *lv, int l0, int L, int nb, int pre, int crs, double omega, int singular,
                  const T *E, const T *N, const T *R, const T *D, T *x, T *b, const MfTab<T> &mf,
                  long start, long span, const CoarseDirect<T> &cd, cudaStream_t st);
// dst[0..n) = src[0..n) (device arrays)
template <typename T> void launch_copy_range(const T *src, T *dst, long n, cudaStream_t st);
// one red-black sweep (both colours) of a one-block level through shared-memory
// tiles, xin -> xout, separable couplings (k_rb_tile); n: the block's points incl. ghosts
template <typename T>
void launch_rb_tile(const BlkDev *blk, const int n[3], double omega, const T *xin, T *xout, const T *b,
                    const PushDev *push, const MfTab<T> &mf, cudaStream_t st);
// the bottom level's couplings, point elements and ghost sources (k_coarse_ops)
template <typename T>
void launch_coarse_ops(const VLev *lv, int lev, int nb, long base, long len, const T *E, const T *N, const T *R,
                       const T *D, const MfTab<T> &mf, float *tag, float *ops, long *elem, cudaStream_t st);
// shared memory the coarse tail may use for its slice of the multigrid arrays
constexpr size_t kVtailSmem = 200 * 1024;
bool prepare_vtail();
bool prepare_rb_tile();  // k_rb_tile's shared memory (false: not usable)
template <typename T>
void launch_mf_tables(const BlkDev *blk, int nb, long maxcell, long max2d, int maxn2, const T *E,
                      const T *N, const T *R, const T *D, const MfTab<T> &t, double tol, int *bad,
                      cudaStream_t st);
template <typename T>
void launch_prolong_fast(const BlkDev *bc, const BlkDev *bf, int nb, const int maxn_f[3], const T *xc,
                         T *xf, const PushDev *push, bool wide, ZMap zm_c, cudaStream_t st);
template <typename T>
void launch_halo_fast(const FaceDev *faces, int nface, long maxface, T *x, cudaStream_t st);
template <typename T>
void launch_resid_outer(const BlkDev *blk, int nb, long maxrow, const double *E, const double *N,
                        const double *R, const double *P, const double *x, const double *b,
                        const double *shift, T *rT, double *r64, double *partial, double *out2,
                        cudaStream_t st);
// one flexible-CG update around a V-cycle whose correction is z: new
// direction p, q = A p, then x += alpha p, r -= alpha q, rT = r; sc[0..3]
// device scalars (sc[2] = 0 restarts), out_rr[0] = r.r
template <typename T>
void launch_fcg(const BlkDev *blk, int nb, long maxcell, const double *E, const double *N, const double *R,
                const double *P, const T *z, double *x, double *pd, double *q, double *r, T *rT,
                const PushDev *push, double *partial, double *sc, double *out_rr, cudaStream_t st);
// out[b] = interior mean of the level-1 field over block b's component
void launch_interior_mean(const BlkDev *blk, int nb, long maxcell, const double *b, double *partial,
                          double *out, cudaStream_t st);
template <typename T>
void launch_update(const BlkDev *blk, int nb, const int maxn[3], double *p, const T *e, const PushDev *push,
                   bool wide, ZMap zm, cudaStream_t st);
template <typename T>
void launch_coarse_mean(const BlkDev *blk, int nb, T *b, cudaStream_t st);

// k_virtbc.cu
void launch_vbc_side(const BlkDev *blk, int nb, int iva, int side, unsigned long long wallmask,
                     unsigned long long initmask, const VbcArgs &a, long maxpts, double visc,
                     double kappa, double aplus, double ylam, double value, cudaStream_t st);

// k_fast.cu: tables of the fast physics kernels.  dst[t][e] = 1 / src[t][e]
// for the first n entries of each table; and the split filter width
// d2[e] = (dip djp rp)^0.33333333 over n2 entries, d1[e] = dkp^0.33333333
// over n1 entries.
void launch_recip(const double *const *src, double *const *dst, int ntab, long n, cudaStream_t st);
void launch_to_f32(const double *const *src, float *const *dst, int ntab, long n, cudaStream_t st);
void launch_delta_tables(const double *dip, const double *djp, const double *rp, long n2,
                         const double *dkp, long n1, double *d2, double *d1, cudaStream_t st);

// k_adjoint.cu: linearised predictors (mode 0 tangent, 1 adjoint pass for
// slot q0, 2 forward value) and the transposes of the linear step operators
void launch_upred_lin(const BlkDev *blk, int nb, long maxcell, int iva, int mode, int q0, const UIntArgs &a,
                      const PredRefs &base, const PredRefs &tan, const PredBars &bar, const double *lam_u,
                      const double *lam_h, double *out_u, double *out_h, double dtime, double visc,
                      double ylaminar, double kappa, double cwfun, cudaStream_t st);
void launch_wpred_lin(const BlkDev *blk, int nb, long maxcell, int mode, int q0, const WIntArgs &a,
                      const PredRefs &base, const PredRefs &tan, const PredBars &bar, const double *lam_u,
                      const double *lam_h, double *out_u, double *out_h, double dtime, double visc,
                      double ylaminar, double kappa, double cwfun, cudaStream_t st);
void launch_take(const BlkDev *blk, int nb, long maxcell, int which, const double *src, double *dst,
                 double *zero_src, cudaStream_t st);
void launch_halo_t(const FaceDev *faces, int nface, long maxface, double *bar, double *wbar, cudaStream_t st);
void launch_extrap_p_t(const BlkDev *blk, int nb, double *bar, cudaStream_t st);
void launch_pref_t(const BlkDev *blk, double *bar, long n, cudaStream_t st);
void launch_sour_p_t(const BlkDev *blk, int nb, long maxcell, double dtime, const double *rdiv,
                     const double *rdju, const double *didjp, const double *dkp, const double *rhonp1,
                     const double *sbar, double *ubar, double *vbar, double *wbar, cudaStream_t st);
void launch_uvw_adv_t(const BlkDev *blk, int nb, long maxcell, int ivar, double dtime, const double *dg,
                      const double *rp, const double *dkw, double *ubar, double *uibar, const double *rho,
                      double *pbar, cudaStream_t st);
void launch_wall_shear(const BlkDev *blk, int nb, long maxik, const double *dju, double visc, const double *u,
                       double coef, double *ubar, double *sum, cudaStream_t st);
void launch_fill_d(double *a, double v, long n, cudaStream_t st);
// linearised Smagorinsky (mode 0 tangent into out, mode 1 pass q0 of 30;
// base/tan/bar fields: u, v, w) and the wall ghosts of set_virt_bc for u and
// w on WALL y sides (mode 0 tangent, 1 transpose)
void launch_sgs_lin(const BlkDev *blk, int nb, long maxcell, int mode, int q0, const PredRefs &base,
                    const PredRefs &tan, const PredBars &bar, const double *lam, double *out, const double *dip,
                    const double *djp, const double *dkp, const double *hijp, const double *hjip, const double *vdd,
                    double csles, cudaStream_t st);
void launch_vbc_lin(const BlkDev *blk, int nb, long maxik, int mode, double *fu, double *fw, const double *tws_u,
                    const double *twn_u, const double *tws_w, const double *twn_w, const long *off_ki,
                    const double *dju, const double *djp, const double *rho, double visc, double ylam,
                    cudaStream_t st);

// k_outflow.cu: convective outflow / fixed inflow sides
void launch_side_flux(const SideJob *jobs, int njobs, int iva, int which, const double *u, const double *v,
                      const double *w, const double *rho, const double *rdju, const double *rdiv,
                      const double *didjp, const double *dkp, double *out, cudaStream_t st);
void launch_side_combine(const SideJob *jobs, int njobs, const double *out, int mode, double *ex,
                         cudaStream_t st);
void launch_exit_update(const SideJob *jobs, int njobs, int task, int iva, const ExitMetrics &M, double *u,
                        double *u_int, const double *rho, const double *rhonp1, double *hn, double dtime,
                        const double *ex, cudaStream_t st);
void launch_exit_scale(const SideJob *jobs, int njobs, int iva, double *f, const double *ex, cudaStream_t st);
void launch_mass_change(const BlkDev *blk, int nb, long maxcell, double dtime, const double *rho,
                        const double *rhonp1, const double *rdidjp, const double *dkw, double *partial,
                        double *out, cudaStream_t st);
void launch_fixed_inlet(const BlkDev *blk, int iblk, int which, int nplane, const double *uprof,
                        const double *vprof, unsigned long long seed, int step, const int *step_dev, double rholo,
                        double rhohi, double *u, double *v, double *w, double *sc1, double *rho, double *u_int,
                        double *v_int, double *w_int, cudaStream_t st);

void launch_statistics(const BlkDev *blk, int nb, long maxpts, long maxij, int no_sam, const double *u,
                       const double *v, const double *w, const double *p, const double *rho, const double *sc1,
                       const double *sc1var, const double *gam, double *ut, double *vt, double *wt,
                       const StatOut &O, cudaStream_t st);
void launch_recycling(const BlkDev *blk, const int *nijk, int nb, int step, int inblock, int jmult, double rhohi,
                      const RecycProf &P, double *u, double *v, double *w, double *sc1, double *rho, double *u_int,
                      double *v_int, double *w_int, double *work, cudaStream_t st);

// whole-step graph: the fast solve's cycle loop controlled on the device
// (k_graph.cu; d_loop layout there)
void launch_loop_init(cudaGraphConditionalHandle h, const double *small, double *loop, double rtol,
                      cudaStream_t st);
void launch_loop_step(cudaGraphConditionalHandle h, const double *small, double *loop, double rtol, int maxit,
                      int may_switch, cudaStream_t st);
void launch_loop_gate(cudaGraphConditionalHandle h, const double *small, double *loop, double rtol, int confirm,
                      cudaStream_t st);
// lester_step's initial pressure for the fast solves (k_graph.cu: k_p_guess)
void launch_p_guess(double *p, double *pp, long n, int istep, const int *istep_dev, int *saved, cudaStream_t st);
void launch_copy_flag(const int *src, double *dst, cudaStream_t st);

} // namespace les

// k_phys.cu and k_sgs.cu, built twice (phys_variant.h): les_exact and les_fast
#define LES_PHYS_LAUNCHERS                                                                          \
    void launch_set_u_int(const BlkDev *blk, int nb, long maxcell, int iva, const UIntArgs &a,      \
                          double dtime, int iststep, double visc, double ylaminar, double kappa,   \
                          double cwfun, cudaStream_t st);                                           \
    void launch_set_w_int(const BlkDev *blk, int nb, long maxcell, const WIntArgs &a, double dtime, \
                          int iststep, double visc, double ylaminar, double kappa, double cwfun,   \
                          cudaStream_t st);                                                         \
    void launch_fill(double *a, double val, long n, cudaStream_t st);                               \
    void launch_face_bc(const BlkDev *blk, int nb, long maxface, int mode, double *f, double *gam,  \
                        double *gaml, const double *sc1, const double *diu, const double *djv,      \
                        const double *rp, const double *dkp, double *grad, long gstride, int gm,    \
                        cudaStream_t st);                                                           \
    void launch_sc1_waves(const BlkDev *blk, int nb, long maxjk, int smin, int smax,                \
                          const Sc1Args &a, double dtime, cudaStream_t st);                         \
    int sc1_sweep_max_ctas(int smem);                                                               \
    cudaError_t launch_sc1_sweep(const BlkDev *blk, const int *cum, const int2 *slice, int nslice,  \
                                 int nctas, int smin, int smax, const Sc1Args &a, double dtime,     \
                                 WaveSync *ws, long limit, cudaStream_t st);                        \
    void launch_sc1var(const BlkDev *blk, int nb, long maxcell, const double *sc1, double *sc1var,  \
                       const double *dip, const double *djp, const double *rp, const double *dkp,   \
                       const double *dkw, const SgsFast &f, cudaStream_t st);                       \
    void launch_subgrid(const BlkDev *blk, int nb, long maxcell, int model, double csles,           \
                        int gotrad, double alpha, double *gam, double *gamsc1, const double *u, const double *v,  \
                        const double *w, const double *sc1, double *sc1var, double *sc1dis,         \
                        const double *vdd, const double *const *m, const SgsFast &f,               \
                        cudaStream_t st);

namespace les_exact {
LES_PHYS_LAUNCHERS
}
namespace les_fast {
LES_PHYS_LAUNCHERS
}
namespace les_f32 {
LES_PHYS_LAUNCHERS
}

// k_sweep.cu: the tiled scalar sweep, built per physics variant (FP64
// exact and fast on FP64 skewed copies, FP32 on FP32 copies)
#define LES_SWEEP_LAUNCHERS(S)                                                                      \
    void launch_sweep_skew(const SkewBlk *sb, int nb, int maxn0, int maxn1, int maxn2, int nfield, \
                           const SkewPtrs<S> &P, int two_d, cudaStream_t st);                      \
    void launch_sweep_unskew(const SkewBlk *sb, int nb, int maxn0, int maxn1, int maxn2,           \
                             const S *sks, const S *skh, double *sc1, double *hsc1,                \
                             cudaStream_t st);                                                      \
    void launch_sweep_init_new(const SkewBlk *sb, int nb, const S *old, S *nw, cudaStream_t st);    \
    int sweep_tiles_smem(int sw);                                                                   \
    int sweep_tiles_max_ctas(int sw, int nthr);                                                     \
    cudaError_t launch_sweep_tiles(const SweepArgs<S> &a, double dtime, long limit, int nctas,     \
                                   int nthr, cudaStream_t st);

namespace les_exact {
LES_SWEEP_LAUNCHERS(double)
}
namespace les_fast {
LES_SWEEP_LAUNCHERS(double)
}
namespace les_f32 {
LES_SWEEP_LAUNCHERS(float)
}
