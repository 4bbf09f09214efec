// lester_adjoint.cu -- adjoint and tangent-linear runs of the time step
// (C ABI: lester_adjoint_run, lester_tangent_run).
//
// Objective: J = mean over steps j_first..j_last of the mean wall shear
// stress visc * u / (0.5 dju) at the wall points of the y sides, for a
// run of nsteps lester_step calls from the given state.  Control: the body
// force per unit volume of lester_gpu_set_body_force.
//
// The adjoint is the exact transpose of the discrete step as lester_step
// computes it, for the flows where that step is smooth in the velocities:
// constant density, no eddy viscosity or the Smagorinsky model (model 1,
// walls on the y sides only, Cartesian), no slip sides, wall points in the
// laminar branch of the wall function, and a converged fast pressure
// solve.  Per step, in reverse order of the forward operations:
//   face copies of u, v, w  ->  uvw_adv  ->  p_ref_subtract, face copies
//   and extrap_p of p  ->  Poisson solve (the matrix is symmetric: the same
//   solver)  ->  sour_p  ->  face copies of u_int, v_int, w_int  ->  the
//   three predictors (local Jacobian rows by forward-mode duals, scattered)
//   ->  with model 1: face copies of gam  ->  Smagorinsky gam (duals)  ->
//   set_virt_bc's wall ghosts of u and w.
// With model 1 the van Driest damping is a constant of the step:
// set_virt_bc resets it to 1 on each of its three calls and the w call's
// wall planes keep the larger of 1 and the van Driest value.  The running
// means of the wall stress then enter only through the branch choices of
// the wall function and the wall ghosts (laminar here).
// Without a model, ghost values of u, v, w on the wall sides enter the
// predictors only multiplied by the zero wall-normal velocity, so their
// adjoints are dropped.
//
// Memory: the state is checkpointed every cfg->checkpoint steps and each
// segment is recomputed forward, keeping its per-step states, before its
// adjoint steps run.
#include <cmath>
#include <cstring>
#include <vector>

#include "kernels.h"
#include "lester_ctx.h"

using namespace les;

namespace {

enum { M_DIP, M_DIU, M_DIV, M_DIX, M_RDIP, M_RDIV, M_RDIX, M_DJP, M_DJU, M_DJV, M_DJX, M_RDJP, M_RDJU,
       M_RDJX, M_HIJP, M_HJIP, M_HKIP, M_HKJP, M_HIJU, M_HJIU, M_HKIU, M_HKJU, M_HIJV, M_HJIV, M_HKIV, M_HKJV,
       M_RP, M_RU, M_RV, M_DIDJP, M_RDIDJP, M_DIDJU, M_RDIDJU, M_DJDIV, M_RDJDIV };

// the step's carried state and scratch, as members of lester_fields
struct Slot {
    double *lester_fields::*m;
    int kind;  // 0: level-1 3-D, 1: all-level 3-D, 2..: wall array q
};

const Slot kCarried[] = {
    {&lester_fields::u, 0},      {&lester_fields::v, 0},       {&lester_fields::w, 0},
    {&lester_fields::sc1, 0},    {&lester_fields::rho, 0},     {&lester_fields::rhonp1, 0},
    {&lester_fields::rhonm1, 0}, {&lester_fields::hn_u, 0},    {&lester_fields::hn_v, 0},
    {&lester_fields::hn_w, 0},   {&lester_fields::hn_sc1, 0},  {&lester_fields::gam, 0},
    {&lester_fields::gamsc1, 0}, {&lester_fields::gamlam, 0},  {&lester_fields::sc1var, 0},
    {&lester_fields::sc1dis, 0}, {&lester_fields::vd_damping, 0}, {&lester_fields::temperature, 0},
    {&lester_fields::p, 1}};
const Slot kScratch[] = {{&lester_fields::u_int, 0},     {&lester_fields::v_int, 0},
                         {&lester_fields::w_int, 0},     {&lester_fields::drhonp1dt, 0},
                         {&lester_fields::srhot, 0},     {&lester_fields::srhoux, 0},
                         {&lester_fields::s, 1},         {&lester_fields::res, 1}};
constexpr int kNCarried = sizeof(kCarried) / sizeof(kCarried[0]);
constexpr int kNScratch = sizeof(kScratch) / sizeof(kScratch[0]);

long wall_len(const Ctx &c, int q)
{
    const long t[12] = {c.totki, c.totki, c.tot2_l1, c.tot2_l1, c.totjk, c.totjk,
                        c.tot2_l1, c.tot2_l1, c.totjk, c.totjk, c.totki, c.totki};
    return t[q];
}

long slot_len(const Ctx &c, int kind) { return kind == 0 ? c.tot_sg3 : c.tot3; }

// device copies of the carried state (18 + p + 12 wall arrays)
struct StateBuf {
    std::vector<double *> a;
};

struct Run {
    Ctx &c;
    lester_fields W{};          // the working fields (work copies + caller's read-only arrays)
    std::vector<double *> own;  // every buffer allocated here
    explicit Run(Ctx &cc) : c(cc) {}
    ~Run()
    {
        for (double *p : own) cudaFree(p);
    }
    int alloc(long n, double **p)
    {
        if (cudaMalloc(p, sizeof(double) * n) != cudaSuccess) {
            cudaGetLastError();
            return set_err(LES_ERR_NOMEM, "adjoint: device allocation of %ld doubles", n);
        }
        own.push_back(*p);
        LES_CUDA(cudaMemsetAsync(*p, 0, sizeof(double) * n, c.stream));
        return 0;
    }
    int alloc_state(StateBuf &s)
    {
        s.a.assign(kNCarried + 12, nullptr);
        int r;
        for (int q = 0; q < kNCarried; q++)
            if ((r = alloc(slot_len(c, kCarried[q].kind), &s.a[q]))) return r;
        for (int q = 0; q < 12; q++)
            if ((r = alloc(wall_len(c, q), &s.a[kNCarried + q]))) return r;
        return 0;
    }
    // dst <- the working state (save) or the working state <- src (load)
    int xfer(StateBuf &s, bool save)
    {
        for (int q = 0; q < kNCarried; q++) {
            double *w = W.*(kCarried[q].m);
            size_t nb = sizeof(double) * slot_len(c, kCarried[q].kind);
            LES_CUDA(cudaMemcpyAsync(save ? s.a[q] : w, save ? w : s.a[q], nb, cudaMemcpyDeviceToDevice, c.stream));
        }
        for (int q = 0; q < 12; q++) {
            size_t nb = sizeof(double) * wall_len(c, q);
            LES_CUDA(cudaMemcpyAsync(save ? s.a[kNCarried + q] : W.tw[q], save ? W.tw[q] : s.a[kNCarried + q], nb,
                                     cudaMemcpyDeviceToDevice, c.stream));
        }
        return 0;
    }
    // working fields: copies of the caller's state and scratch, the caller's
    // coefficients and metrics
    int setup(const lester_fields &F)
    {
        W = F;
        int r;
        for (int q = 0; q < kNCarried; q++) {
            double *d;
            long n = slot_len(c, kCarried[q].kind);
            if ((r = alloc(n, &d))) return r;
            const double *src = F.*(kCarried[q].m);
            if (!src) return set_err(LES_ERR_ARG, "adjoint: state array %d is NULL", q);
            LES_CUDA(cudaMemcpyAsync(d, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
            W.*(kCarried[q].m) = d;
        }
        for (int q = 0; q < kNScratch; q++) {
            double *d;
            if ((r = alloc(slot_len(c, kScratch[q].kind), &d))) return r;
            W.*(kScratch[q].m) = d;
        }
        for (int q = 0; q < 12; q++) {
            double *d;
            if ((r = alloc(wall_len(c, q), &d))) return r;
            if (!F.tw[q]) return set_err(LES_ERR_ARG, "adjoint: wall array %d is NULL", q);
            LES_CUDA(cudaMemcpyAsync(d, F.tw[q], sizeof(double) * wall_len(c, q), cudaMemcpyDeviceToDevice,
                                     c.stream));
            W.tw[q] = d;
        }
        return 0;
    }
};

int check_device(const lester_fields &F)
{
    const double *all[] = {F.u, F.v, F.w, F.p, F.ap, F.metric[0], F.dkp, F.tw[0]};
    for (const double *p : all) {
        cudaPointerAttributes at;
        if (!p || cudaPointerGetAttributes(&at, p) != cudaSuccess ||
            (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
            cudaGetLastError();
            return set_err(LES_ERR_ARG, "adjoint: the fields must be device arrays");
        }
    }
    return 0;
}

int check_scope(const Ctx &c, const lester_adj_cfg &cfg)
{
    const lester_ctrl &k = c.c;
    if (k.psolve == LES_PSOLVE_REFERENCE)
        return set_err(LES_ERR_ARG, "adjoint: needs a converged fast pressure solve (psolve FP64 or MIXED)");
    if (k.rholo != k.rhohi) return set_err(LES_ERR_ARG, "adjoint: constant density only (rholo == rhohi)");
    if (k.phys32 && !k.exact)
        return set_err(LES_ERR_ARG, "adjoint: the linearised step is FP64; phys32 must be 0");
    if (k.model != 0 && k.model != 1)
        return set_err(LES_ERR_ARG, "adjoint: no eddy viscosity (model 0) or Smagorinsky (model 1) only");
    if (k.model == 1) {
        if (c.g.gotrad) return set_err(LES_ERR_ARG, "adjoint: Smagorinsky on Cartesian grids only");
        for (int b = 0; b < c.g.numbl; b++)
            for (int s = 0; s < 6; s++) {
                const int bc = c.g.bl_bc[b][s];
                const bool open = bc == LES_BCT_PERIODIC || bc == LES_BCT_INTERFACE;
                if (!open && !(bc == LES_BCT_WALL && (s == 2 || s == 3)))
                    return set_err(LES_ERR_ARG, "adjoint: Smagorinsky with walls on the y sides only");
            }
    }
    for (int b = 0; b < c.g.numbl; b++)
        for (int s = 0; s < 6; s++)
            if (c.g.bl_bc[b][s] == LES_BCT_ZERO_GRAD)
                return set_err(LES_ERR_ARG, "adjoint: slip (zero-gradient) sides are not supported");
    if (cfg.nsteps < 1 || cfg.j_first < 1 || cfg.j_last < cfg.j_first || cfg.j_last > cfg.nsteps ||
        cfg.checkpoint < 1)
        return set_err(LES_ERR_ARG, "adjoint: bad run configuration");
    return 0;
}

long wall_points(const Ctx &c)
{
    long n = 0;
    for (int b = 1; b <= c.g.numbl; b++)
        for (int s = 2; s < 4; s++)
            if (c.g.bl_bc[b - 1][s] == LES_BCT_WALL)
                n += (long)(c.lv[1].n[b][0] - 2) * (c.lv[1].n[b][2] - 2);
    return n;
}

long max_ik(const Ctx &c)
{
    long m = 0;
    for (int b = 1; b <= c.g.numbl; b++)
        m = std::max(m, (long)(c.lv[1].n[b][0] - 2) * (c.lv[1].n[b][2] - 2));
    return m;
}

// sum of visc u / (0.5 dju) over the wall points (and its gradient times coef into ubar)
int wall_shear(Ctx &c, const lester_fields &W, const double *u, double coef, double *ubar, double *sum_out)
{
    LES_CUDA(cudaMemsetAsync(c.d_small + 40, 0, sizeof(double), c.stream));
    launch_wall_shear(c.lv[1].d_blk, c.g.numbl, max_ik(c), W.metric[M_DJU], c.c.visc, u, coef, ubar,
                      sum_out ? c.d_small + 40 : nullptr, c.stream);
    if (sum_out) {
        LES_CUDA(cudaMemcpyAsync(c.h_small + 40, c.d_small + 40, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        LES_CUDA(cudaStreamSynchronize(c.stream));
        *sum_out = c.h_small[40];
    }
    return 0;
}

int do_step(Ctx &c, lester_fields &W, int istep)
{
    int r = lester_step(&W, &istep);
    if (r) return r;  // not converged counts as an error here
    return 0;
}

UIntArgs uargs(Ctx &c, const lester_fields &B, int iva)
{
    UIntArgs A;
    memset(&A, 0, sizeof A);
    double *const *m = B.metric;
    const double *mu1[20] = {m[M_DIP], m[M_DIU], m[M_DIX], m[M_RDIX], m[M_DJP], m[M_DJU], m[M_DJV],
                             m[M_DJX], m[M_RDJP], m[M_RDJU], m[M_DIDJP], m[M_DIDJU], m[M_RDIDJU],
                             m[M_HIJP], m[M_HIJU], m[M_HJIU], m[M_HKIU], m[M_HKJU], m[M_RP], m[M_RU]};
    const double *mu2[20] = {m[M_DJP], m[M_DJV], m[M_DJX], m[M_RDJX], m[M_DIP], m[M_DIV], m[M_DIU],
                             m[M_DIX], m[M_RDIP], m[M_RDIV], m[M_DIDJP], m[M_DJDIV], m[M_RDJDIV],
                             m[M_HJIP], m[M_HJIV], m[M_HIJV], m[M_HKJV], m[M_HKIV], m[M_RP], m[M_RV]};
    const double **md[20] = {&A.dip, &A.diu, &A.dix, &A.rdix, &A.djp, &A.dju, &A.djv, &A.djx, &A.rdjp,
                             &A.rdju, &A.didjp, &A.didju, &A.rdidju, &A.hijp, &A.hiju, &A.hjiu, &A.hkiu,
                             &A.hkju, &A.rp, &A.ru};
    for (int q = 0; q < 20; q++) *md[q] = iva == 1 ? mu1[q] : mu2[q];
    A.dkp = B.dkp;
    A.dkw = B.dkw;
    A.rho = B.rho;
    A.rhonp1 = B.rhonp1;
    A.gam = B.gam;
    A.tw_s = B.tw[iva == 1 ? 0 : 4];
    A.tw_n = B.tw[iva == 1 ? 1 : 5];
    A.tw_l = B.tw[iva == 1 ? 2 : 6];
    A.tw_r = B.tw[iva == 1 ? 3 : 7];
    A.off_ki = c.d_offki;
    A.off_jk = c.d_offjk;
    A.off2_lev1_base = 0;
    return A;
}

WIntArgs wargs(Ctx &c, const lester_fields &B)
{
    WIntArgs A;
    memset(&A, 0, sizeof A);
    double *const *m = B.metric;
    const double *mu[MW_N] = {m[M_DIP], m[M_DIU], m[M_RDIV], m[M_DJP], m[M_DJV], m[M_RDJU], m[M_DIDJP],
                              m[M_RDIDJP], m[M_HKIP], m[M_HKJP], m[M_HKIU], m[M_HKJV], m[M_RP], m[M_RU]};
    for (int q = 0; q < MW_N; q++) A.m[q] = mu[q];
    A.dkp = B.dkp;
    A.dkw = B.dkw;
    A.rho = B.rho;
    A.rhonp1 = B.rhonp1;
    A.gam = B.gam;
    A.tw_sfk = B.tw[10];
    A.tw_nfk = B.tw[11];
    A.tw_wfk = B.tw[8];
    A.tw_efk = B.tw[9];
    A.off_ki = c.d_offki;
    A.off_jk = c.d_offjk;
    return A;
}

// the base fields B (state before the step) seen as a lester_fields
lester_fields base_fields(const lester_fields &W, const StateBuf &s)
{
    lester_fields B = W;
    for (int q = 0; q < kNCarried; q++) B.*(kCarried[q].m) = s.a[q];
    for (int q = 0; q < 12; q++) B.tw[q] = s.a[kNCarried + q];
    return B;
}

// zero the ghost planes of the non-periodic sides (set_virt_bc rewrites them)
__global__ void k_zero_wall_ghosts(const BlkDev *__restrict__ blk, double *__restrict__ a)
{
    const BlkDev b = blk[blockIdx.y];
    const int side = blockIdx.z;
    int bc = b.bc[side];
    if (bc == LES_BCT_PERIODIC_D || bc == LES_BCT_INTERFACE_D) return;
    int d = side / 2, hi = side & 1;
    int n0 = b.n[0], n1 = b.n[1], n2 = b.n[2];
    int na = d == 0 ? n1 : n0, nb2 = d == 2 ? n1 : n2;
    long n = (long)na * nb2;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        int x = (int)(q % na), y = (int)(q / na);
        int c0 = hi ? (d == 0 ? n0 : d == 1 ? n1 : n2) - 1 : 0;
        int i = d == 0 ? c0 : x, j = d == 1 ? c0 : (d == 0 ? x : y), k = d == 2 ? c0 : y;
        a[b.off3 + i + (long)n0 * (j + (long)n1 * k)] = 0.;
    }
}

// the linearisation point of a step with the Smagorinsky model: the
// velocities after set_virt_bc, the damping and eddy viscosity of the step
// (and subgrid's other outputs, unused)
struct Lin {
    double *u, *v, *w, *vdd, *gam, *gsc, *svar, *sdis;
};

// zero the interior points of every block
__global__ void k_zero_interior(const BlkDev *__restrict__ blk, double *__restrict__ a)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    a[decode_interior(b, q, i, j, k)] = 0.;
}

struct Adj {
    double *ub, *vb, *wb, *pb, *hub, *hvb, *hwb;   // adjoint of the carried state
    double *uib, *vib, *wib;                       // adjoint of u_int, v_int, w_int
    double *lam_h[3];                              // adjoint of the new h (taken)
    double *bsolve, *xsolve, *res;                 // adjoint Poisson solve (all levels)
    double *wbar;                                  // face-copy buffer
    double *gamb;                                  // model 1: adjoint of gam (carried)
    Lin S;
};

bool smagorinsky(const Ctx &c) { return c.c.model == 1; }

// the step's wall ghosts, damping and eddy viscosity from the state B, as
// lester_step computes them, into S
int base_physics(Ctx &c, const lester_fields &B, Lin &S)
{
    const size_t nb = sizeof(double) * c.tot_sg3;
    LES_CUDA(cudaMemcpyAsync(S.u, B.u, nb, cudaMemcpyDeviceToDevice, c.stream));
    LES_CUDA(cudaMemcpyAsync(S.v, B.v, nb, cudaMemcpyDeviceToDevice, c.stream));
    LES_CUDA(cudaMemcpyAsync(S.w, B.w, nb, cudaMemcpyDeviceToDevice, c.stream));
    LES_CUDA(cudaMemcpyAsync(S.gam, B.gam, nb, cudaMemcpyDeviceToDevice, c.stream));
    double *const *m = B.metric;
    double *const *tw = B.tw;
    const int one = 1;
    double zero = 0.0;
    int r;
    for (int iv = 1; iv <= 3; iv++) {
        double *fld = iv == 1 ? S.u : iv == 2 ? S.v : S.w;
        if ((r = lester_set_virt_bc(&iv, &one, fld, nullptr, B.rho, S.gam, S.vdd, nullptr, &zero, tw[0], tw[1],
                                    tw[2], tw[3], tw[4], tw[5], tw[6], tw[7], tw[8], tw[9], tw[10], tw[11], m[M_DIP],
                                    m[M_DIU], m[M_DIV], m[M_DIX], m[M_DJP], m[M_DJU], m[M_DJV], m[M_DJX], m[M_RU],
                                    m[M_RV], B.dkp, B.dkw)))
            return r;
    }
    return lester_subgrid(S.gam, S.gsc, S.u, S.v, S.w, B.sc1, B.rho, S.svar, S.sdis, S.vdd, m[M_DIP], m[M_DIU],
                          m[M_DJP], m[M_DJV], B.dkp, B.dkw, m[M_HIJP], m[M_HJIP], m[M_HKIP], m[M_HKJP], m[M_RP],
                          nullptr, nullptr);
}

void vbc_lin(Ctx &c, const lester_fields &B, int mode, double *fu, double *fw)
{
    LevelGeom &L = c.lv[1];
    double *const *m = B.metric;
    launch_vbc_lin(L.d_blk, c.g.numbl, max_ik(c), mode, fu, fw, B.tw[0], B.tw[1], B.tw[10], B.tw[11], c.d_offki,
                   m[M_DJU], m[M_DJP], B.rho, c.c.visc, c.c.ylaminar, c.stream);
}

int halo_t(Ctx &c, double *bar, double *wbar)
{
    LevelGeom &L = c.lv[1];
    launch_halo_t(L.d_face, L.nface, L.maxface, bar, wbar, c.stream);
    return 0;
}

void zero_wall_ghosts(Ctx &c, double *a)
{
    LevelGeom &L = c.lv[1];
    long m = 0;
    for (int b = 1; b <= c.g.numbl; b++) {
        const int *n = L.n[b];
        m = std::max(m, std::max((long)n[1] * n[2], std::max((long)n[0] * n[2], (long)n[0] * n[1])));
    }
    unsigned gx = (unsigned)((m + 255) / 256);
    k_zero_wall_ghosts<<<dim3(gx, c.g.numbl, 6), 256, 0, c.stream>>>(L.d_blk, a);
    count_launch(1);
}

constexpr int kSlotsU = 19, kSlotsW = 19;  // inputs of the u/v and w predictors (k_adjoint.cu)

// one adjoint step: A holds the adjoint of the state after step n; on
// return, of the state before it.  B is that state (the linearisation
// point); gf[] accumulate the body-force gradient.
int adjoint_step(Ctx &c, const lester_fields &W, const lester_fields &B, Adj &A, double *const gf[3])
{
    LevelGeom &L = c.lv[1];
    const int nb = c.g.numbl;
    const lester_ctrl &k = c.c;
    double *const *m = W.metric;
    int r;
    // projection: face copies then uvw_adv, per component
    LES_CUDA(cudaMemsetAsync(A.uib, 0, sizeof(double) * c.tot_sg3, c.stream));
    LES_CUDA(cudaMemsetAsync(A.vib, 0, sizeof(double) * c.tot_sg3, c.stream));
    LES_CUDA(cudaMemsetAsync(A.wib, 0, sizeof(double) * c.tot_sg3, c.stream));
    double *ubs[3] = {A.ub, A.vb, A.wb}, *uis[3] = {A.uib, A.vib, A.wib};
    const double *dg[3] = {m[M_DIU], m[M_DJV], m[M_DIU]};
    for (int iv = 3; iv >= 1; iv--) {
        halo_t(c, ubs[iv - 1], A.wbar);
        launch_uvw_adv_t(L.d_blk, nb, L.maxcell, iv, k.dtime, dg[iv - 1], m[M_RP], W.dkw, ubs[iv - 1],
                         uis[iv - 1], B.rhonp1, A.pb, c.stream);
    }
    // pressure: p_ref_subtract, face copies, extrap_p, then the solve (the
    // matrix is symmetric: its transpose is solved by the same solver)
    launch_pref_t(L.d_blk, A.pb, c.tot_sg3, c.stream);
    halo_t(c, A.pb, A.wbar);
    launch_extrap_p_t(L.d_blk, nb, A.pb, c.stream);
    LES_CUDA(cudaMemsetAsync(A.bsolve, 0, sizeof(double) * c.tot3, c.stream));
    LES_CUDA(cudaMemsetAsync(A.xsolve, 0, sizeof(double) * c.tot3, c.stream));
    LES_CUDA(cudaMemcpyAsync(A.bsolve, A.pb, sizeof(double) * c.tot_sg3, cudaMemcpyDeviceToDevice, c.stream));
    bool wn = c.want_norms;
    c.want_norms = false;
    r = lester_lmg_solve(W.ap, W.aw, W.ae, W.as, W.an, W.al, W.ar, A.xsolve, A.bsolve, A.res, nullptr, nullptr);
    c.want_norms = wn;
    if (r) return r;
    LES_CUDA(cudaMemsetAsync(A.pb, 0, sizeof(double) * c.tot_sg3, c.stream));
    // sour_p, then the face copies of u_int, v_int, w_int
    launch_sour_p_t(L.d_blk, nb, L.maxcell, k.dtime, m[M_RDIV], m[M_RDJU], m[M_DIDJP], W.dkp, B.rhonp1,
                    A.xsolve, A.uib, A.vib, A.wib, c.stream);
    halo_t(c, A.uib, A.wbar);
    halo_t(c, A.vib, A.wbar);
    halo_t(c, A.wib, A.wbar);
    // predictors: take the adjoints of the new h, then one pass per input slot
    launch_take(L.d_blk, nb, L.maxcell, 1, A.hub, A.lam_h[0], A.hub, c.stream);
    launch_take(L.d_blk, nb, L.maxcell, 2, A.hvb, A.lam_h[1], A.hvb, c.stream);
    launch_take(L.d_blk, nb, L.maxcell, 3, A.hwb, A.lam_h[2], A.hwb, c.stream);
    PredRefs none;
    memset(&none, 0, sizeof none);
    const double *fbase[3] = {c.fb[0], c.fb[1], c.fb[2]};
    // the linearisation point: the state, or with model 1 the velocities
    // after set_virt_bc and the step's eddy viscosity
    const bool sgs = smagorinsky(c);
    const double *bu = B.u, *bv = B.v, *bw = B.w, *bg = nullptr;
    double *gb = nullptr;
    int nsu = kSlotsU, nsw = kSlotsW;
    if (sgs) {
        if ((r = base_physics(c, B, A.S))) return r;
        bu = A.S.u;
        bv = A.S.v;
        bw = A.S.w;
        bg = A.S.gam;
        gb = A.gamb;
        nsu = kSlotsU + 10;
        nsw = kSlotsW + 10;
    }
    {
        UIntArgs a1 = uargs(c, B, 1);
        PredRefs base = {{bu, bv, bw, B.p, B.hn_u, fbase[0], bg}};
        PredBars bar = {{A.ub, A.vb, A.wb, A.pb, A.hub, gf[0], gb}};
        for (int q = 0; q < nsu; q++)
            launch_upred_lin(L.d_blk, nb, L.maxcell, 1, 1, q, a1, base, none, bar, A.uib, A.lam_h[0], nullptr,
                             nullptr, k.dtime, k.visc, k.ylaminar, k.kappa, k.cwfun, c.stream);
    }
    {
        UIntArgs a2 = uargs(c, B, 2);
        PredRefs base = {{bv, bu, bw, B.p, B.hn_v, fbase[1], bg}};
        PredBars bar = {{A.vb, A.ub, A.wb, A.pb, A.hvb, gf[1], gb}};
        for (int q = 0; q < nsu; q++)
            launch_upred_lin(L.d_blk, nb, L.maxcell, 2, 1, q, a2, base, none, bar, A.vib, A.lam_h[1], nullptr,
                             nullptr, k.dtime, k.visc, k.ylaminar, k.kappa, k.cwfun, c.stream);
    }
    {
        WIntArgs aw = wargs(c, B);
        PredRefs base = {{bu, bv, bw, B.p, B.hn_w, fbase[2], bg}};
        PredBars bar = {{A.ub, A.vb, A.wb, A.pb, A.hwb, gf[2], gb}};
        for (int q = 0; q < nsw; q++)
            launch_wpred_lin(L.d_blk, nb, L.maxcell, 1, q, aw, base, none, bar, A.wib, A.lam_h[2], nullptr,
                             nullptr, k.dtime, k.visc, k.ylaminar, k.kappa, k.cwfun, c.stream);
    }
    if (sgs) {
        // gam after its face copies, then the wall ghosts of u and w.  The
        // copies gather every partner plane before writing any ghost plane,
        // so a corner ghost takes the previous step's value at an edge
        // ghost: what the transposed copies leave on ghost points is the
        // adjoint of the previous step's gam there and is carried; the
        // interior (rewritten by subgrid) and the wall ghosts (never
        // written) are cleared.
        halo_t(c, A.gamb, A.wbar);
        PredRefs base = {{bu, bv, bw}};
        PredBars bar = {{A.ub, A.vb, A.wb}};
        for (int q = 0; q < 30; q++)
            launch_sgs_lin(L.d_blk, nb, L.maxcell, 1, q, base, none, bar, A.gamb, nullptr, m[M_DIP], m[M_DJP],
                           W.dkp, m[M_HIJP], m[M_HJIP], A.S.vdd, k.csles, c.stream);
        k_zero_interior<<<dim3((unsigned)((L.maxcell + 255) / 256), nb), 256, 0, c.stream>>>(L.d_blk, A.gamb);
        count_launch(1);
        zero_wall_ghosts(c, A.gamb);
        vbc_lin(c, B, 1, A.ub, A.wb);
    }
    // wall ghosts of the state before the step are rewritten (set_virt_bc)
    zero_wall_ghosts(c, A.ub);
    zero_wall_ghosts(c, A.vb);
    zero_wall_ghosts(c, A.wb);
    LES_CUDA(cudaGetLastError());
    return 0;
}

int alloc_lin(Run &R, Lin &S)
{
    int r;
    double **sg[] = {&S.u, &S.v, &S.w, &S.vdd, &S.gam, &S.gsc, &S.svar, &S.sdis};
    for (double **p : sg)
        if ((r = R.alloc(R.c.tot_sg3, p))) return r;
    return 0;
}

int alloc_adj(Run &R, Adj &A)
{
    Ctx &c = R.c;
    int r;
    memset(&A, 0, sizeof A);
    if (smagorinsky(c)) {
        if ((r = alloc_lin(R, A.S)) || (r = R.alloc(c.tot_sg3, &A.gamb))) return r;
    }
    double **sg[] = {&A.ub, &A.vb, &A.wb, &A.pb, &A.hub, &A.hvb, &A.hwb, &A.uib, &A.vib, &A.wib,
                     &A.lam_h[0], &A.lam_h[1], &A.lam_h[2]};
    for (double **p : sg)
        if ((r = R.alloc(c.tot_sg3, p))) return r;
    double **mg[] = {&A.bsolve, &A.xsolve, &A.res};
    for (double **p : mg)
        if ((r = R.alloc(c.tot3, p))) return r;
    long wl = 0;
    for (int lev = 1; lev <= c.nummgl; lev++) wl = std::max(wl, c.lv[lev].worklen);
    return R.alloc(wl + 16, &A.wbar);
}

} // namespace

extern "C" {

int lester_adjoint_run(const lester_adj_cfg *cfg, const lester_fields *fields, double *J, double *gfu,
                       double *gfv, double *gfw)
{
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    int r;
    if (!cfg || !fields || !J || !gfu || !gfv || !gfw) return set_err(LES_ERR_ARG, "adjoint: NULL argument");
    if ((r = check_scope(c, *cfg)) || (r = check_device(*fields))) return r;
    const int N = cfg->nsteps, K = cfg->checkpoint;
    const int iststep0 = c.iststep;
    Run R(c);
    if ((r = R.setup(*fields))) return r;
    double *gf[3] = {gfu, gfv, gfw};
    for (double *g : gf) LES_CUDA(cudaMemsetAsync(g, 0, sizeof(double) * c.tot_sg3, c.stream));
    const long nw = wall_points(c);
    if (nw == 0) return set_err(LES_ERR_ARG, "adjoint: no wall points on the y sides");
    const double coef = 1.0 / ((double)nw * (cfg->j_last - cfg->j_first + 1));
    const int nseg = (N + K - 1) / K;
    std::vector<StateBuf> chk(nseg), seg(K);
    for (auto &s : chk)
        if ((r = R.alloc_state(s))) return r;
    for (auto &s : seg)
        if ((r = R.alloc_state(s))) return r;
    // forward, with checkpoints
    double jsum = 0;
    for (int n = 1; n <= N; n++) {
        if ((n - 1) % K == 0) R.xfer(chk[(n - 1) / K], true);
        c.iststep = iststep0 + (n - 1);
        if ((r = do_step(c, R.W, n + 1))) break;
        if (n >= cfg->j_first && n <= cfg->j_last) {
            double sm;
            if ((r = wall_shear(c, R.W, R.W.u, 0., nullptr, &sm))) break;
            jsum += coef * sm;
        }
    }
    if (r) {
        c.iststep = iststep0;
        return r;
    }
    *J = jsum;
    // backward, segment by segment
    Adj A;
    if ((r = alloc_adj(R, A))) return r;
    for (int s = nseg - 1; s >= 0 && !r; s--) {
        const int n0 = s * K + 1, n1 = std::min((s + 1) * K, N);
        R.xfer(chk[s], false);
        for (int n = n0; n <= n1 && !r; n++) {
            R.xfer(seg[n - n0], true);
            c.iststep = iststep0 + (n - 1);
            if (n < n1) r = do_step(c, R.W, n + 1);
        }
        for (int n = n1; n >= n0 && !r; n--) {
            if (n >= cfg->j_first && n <= cfg->j_last) r = wall_shear(c, R.W, R.W.u, coef, A.ub, nullptr);
            if (!r) {
                lester_fields B = base_fields(R.W, seg[n - n0]);
                r = adjoint_step(c, R.W, B, A, gf);
            }
        }
    }
    c.iststep = iststep0;
    if (r) return r;
    LES_CUDA(cudaStreamSynchronize(c.stream));
    LES_CUDA(cudaGetLastError());
    return 0;
}

int lester_tangent_run(const lester_adj_cfg *cfg, const lester_fields *fields, const double *dfu,
                       const double *dfv, const double *dfw, double *J, double *dJ)
{
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    int r;
    if (!cfg || !fields || !J || !dJ) return set_err(LES_ERR_ARG, "tangent: NULL argument");
    if ((r = check_scope(c, *cfg)) || (r = check_device(*fields))) return r;
    const int N = cfg->nsteps;
    const int iststep0 = c.iststep;
    Run R(c);
    if ((r = R.setup(*fields))) return r;
    LevelGeom &L = c.lv[1];
    const int nb = c.g.numbl;
    const lester_ctrl &k = c.c;
    double *du, *dv, *dw, *dp, *dpn, *ds, *dres, *dhu, *dhv, *dhw, *dui, *dvi, *dwi, *sc[3];
    double **sg[] = {&du, &dv, &dw, &dhu, &dhv, &dhw, &dui, &dvi, &dwi, &sc[0], &sc[1], &sc[2]};
    for (double **p : sg)
        if ((r = R.alloc(c.tot_sg3, p))) return r;
    double **mg[] = {&dp, &dpn, &ds, &dres};
    for (double **p : mg)
        if ((r = R.alloc(c.tot3, p))) return r;
    // model 1: the linearisation point and the tangent of gam (kept from
    // step to step: its edge ghosts feed the next step's corner ghosts)
    const bool sgs = smagorinsky(c);
    Lin S{};
    double *dgam = nullptr;
    if (sgs && ((r = alloc_lin(R, S)) || (r = R.alloc(c.tot_sg3, &dgam)))) return r;
    const long nw = wall_points(c);
    if (nw == 0) return set_err(LES_ERR_ARG, "tangent: no wall points on the y sides");
    const double coef = 1.0 / ((double)nw * (cfg->j_last - cfg->j_first + 1));
    double *const *m = R.W.metric;
    PredBars nob;
    memset(&nob, 0, sizeof nob);
    double jsum = 0, djsum = 0;
    const int one = 1, two = 2, iv0 = 0;
    for (int n = 1; n <= N && !r; n++) {
        lester_fields &W = R.W;
        const double *fbase[3] = {c.fb[0], c.fb[1], c.fb[2]};
        const double *bu = W.u, *bv = W.v, *bw = W.w, *bg = nullptr;
        if (sgs) {
            // wall ghosts and gam of the step, with their tangents
            if ((r = base_physics(c, W, S))) break;
            bu = S.u;
            bv = S.v;
            bw = S.w;
            bg = S.gam;
            vbc_lin(c, W, 0, du, dw);
            PredRefs base = {{bu, bv, bw}}, tan = {{du, dv, dw}};
            launch_sgs_lin(L.d_blk, nb, L.maxcell, 0, 0, base, tan, nob, nullptr, dgam, m[M_DIP], m[M_DJP], W.dkp,
                           m[M_HIJP], m[M_HJIP], S.vdd, k.csles, c.stream);
            if ((r = lester_swap_sc(&iv0, &one, dgam, nullptr, &two))) break;
        }
        // tangent predictors at the state before the step
        {
            UIntArgs a1 = uargs(c, W, 1);
            PredRefs base = {{bu, bv, bw, W.p, W.hn_u, fbase[0], bg}}, tan = {{du, dv, dw, dp, dhu, dfu, dgam}};
            launch_upred_lin(L.d_blk, nb, L.maxcell, 1, 0, 0, a1, base, tan, nob, nullptr, nullptr, dui, dhu,
                             k.dtime, k.visc, k.ylaminar, k.kappa, k.cwfun, c.stream);
            UIntArgs a2 = uargs(c, W, 2);
            PredRefs base2 = {{bv, bu, bw, W.p, W.hn_v, fbase[1], bg}}, tan2 = {{dv, du, dw, dp, dhv, dfv, dgam}};
            launch_upred_lin(L.d_blk, nb, L.maxcell, 2, 0, 0, a2, base2, tan2, nob, nullptr, nullptr, dvi, dhv,
                             k.dtime, k.visc, k.ylaminar, k.kappa, k.cwfun, c.stream);
            WIntArgs aw = wargs(c, W);
            PredRefs base3 = {{bu, bv, bw, W.p, W.hn_w, fbase[2], bg}}, tan3 = {{du, dv, dw, dp, dhw, dfw, dgam}};
            launch_wpred_lin(L.d_blk, nb, L.maxcell, 0, 0, aw, base3, tan3, nob, nullptr, nullptr, dwi, dhw,
                             k.dtime, k.visc, k.ylaminar, k.kappa, k.cwfun, c.stream);
        }
        // the rest of the step is linear: the step's own operators on the tangents
        if ((r = lester_swap_sc(&iv0, &one, dui, nullptr, &two)) ||
            (r = lester_swap_sc(&iv0, &one, dvi, nullptr, &two)) ||
            (r = lester_swap_sc(&iv0, &one, dwi, nullptr, &two)))
            break;
        if ((r = lester_sour_p(m[M_DIU], m[M_DJV], m[M_RDIV], m[M_RDJU], m[M_DIDJP], W.dkp, m[M_RDIDJP], W.dkw, dui,
                               dvi, dwi, W.rho, W.rhonp1, sc[0], ds, sc[1], sc[2], nullptr, nullptr)))
            break;
        LES_CUDA(cudaMemsetAsync(dpn, 0, sizeof(double) * c.tot3, c.stream));
        bool wn = c.want_norms;
        c.want_norms = false;
        r = lester_lmg_solve(W.ap, W.aw, W.ae, W.as, W.an, W.al, W.ar, dpn, ds, dres, nullptr, nullptr);
        c.want_norms = wn;
        if (r || (r = lester_extrap_p(dpn, nullptr, nullptr)) || (r = lester_p_ref_subtract(dpn))) break;
        const int ivs[3] = {1, 2, 3};
        const double *dg[3] = {m[M_DIU], m[M_DJV], m[M_DIU]};
        double *dvel[3] = {du, dv, dw}, *dint[3] = {dui, dvi, dwi};
        for (int q = 0; q < 3 && !r; q++)
            r = lester_uvw_adv(&ivs[q], dg[q], m[M_RP], W.dkw, dvel[q], dint[q], W.rhonp1, dpn, nullptr, nullptr,
                               &two);
        if (r) break;
        LES_CUDA(cudaMemcpyAsync(dp, dpn, sizeof(double) * c.tot_sg3, cudaMemcpyDeviceToDevice, c.stream));
        // the base step
        c.iststep = iststep0 + (n - 1);
        if ((r = do_step(c, W, n + 1))) break;
        if (n >= cfg->j_first && n <= cfg->j_last) {
            double sm, dsm;
            if ((r = wall_shear(c, W, W.u, 0., nullptr, &sm)) || (r = wall_shear(c, W, du, 0., nullptr, &dsm)))
                break;
            jsum += coef * sm;
            djsum += coef * dsm;
        }
    }
    c.iststep = iststep0;
    if (r) return r;
    *J = jsum;
    *dJ = djsum;
    return 0;
}

} // extern "C"
