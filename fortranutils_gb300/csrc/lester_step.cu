// lester_step.cu -- one LES time step on the device: the ivar loop of
// code/step.F:214-454 (u, v, w, p; the sc1 pass has no work without a
// convective outflow) calling the library's routines in the reference's
// order.  Work the reference does only for output or diagnostics
// (statistics, field output, cflest) and the inflow/outflow routines of
// sides this library does not support (FIXED inlet, CONVECTIVE outflow)
// are not part of it; a block with such a side is refused.
//
// Field pointers may be host or device arrays.  Host arrays cross once each
// way per call at most, on two copy streams beside the compute stream: an
// input's copy is waited for just before the first routine that reads it,
// an output is copied back as soon as the step has written it for the last
// time, so that most of the traffic overlaps the step's kernels.  Scratch
// fields passed as NULL are kept on the device by the library.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
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

// step.F:214-420 up to the Poisson right-hand side: inlet planes, wall
// ghosts, eddy viscosity, scalar, the three predictors, coeff_p (first
// step), sour_p
static int step_pre(Ctx &c, lester_fields &D, const int *istep)
{
    double *const *m = D.metric;
    double **tw = D.tw;
    const lester_ctrl &k = c.c;
    const int one = 1, iU = 1, iV = 2;
    double zero = 0.0;
    const double *mx[12] = {m[M_DIP], m[M_DIU], m[M_DIX], m[M_DJP], m[M_DJV], m[M_DJX],
                            m[M_RDIV], m[M_RDJU], m[M_DIDJP], m[M_RP], m[M_RU], m[M_RV]};
    // conv_exitbc(task, iva) of step.F:344 and 435
    auto exitbc = [&](int task, int iva) {
        return exit_task(c, task, iva, D.rho, D.rhonp1, D.u, D.v, D.w, D.u_int, D.v_int, D.w_int, D.hn_u, D.hn_v,
                         D.hn_w, mx, D.dkp, D.dkw, m[M_RDIDJP]);
    };
    // deferred host copies: wait for inputs, copy outputs back early
    auto need = [&](std::initializer_list<const double *> l) {
        if (c.xfer)
            for (const double *q : l) RET(c.xfer->need(q));
        return 0;
    };
    auto put = [&](std::initializer_list<const double *> l) {
        if (c.xfer)
            for (const double *q : l) RET(c.xfer->put(q));
        return 0;
    };
    if (has_inlet(c))
        RET(need({D.u, D.v, D.w, D.sc1, D.rho}));
    RET(need({D.dkp, D.dkw, D.u, D.rho, D.vd_damping}));
    for (int q = 0; q < 35; q++) RET(need({m[q]}));
    for (int q = 0; q < 12; q++) RET(need({tw[q]}));
    // ---- ivar = u: the inlet planes (step.F:226)
    if (has_inlet(c))
        RET(inlet_task(c, c.d_uprof, c.d_vprof, c.inlet_seed, *istep, D.u, D.v, D.w, D.sc1, D.rho, D.u_int,
                       D.v_int, D.w_int));
    // ---- ivar = u: boundary ghosts, eddy viscosity, scalar, u predictor
    for (int iv = 1; iv <= 3; iv++) {
        double *fld = iv == 1 ? D.u : iv == 2 ? D.v : D.w;
        RET(need({fld}));
        RET(lester_set_virt_bc(&iv, &one, fld, nullptr, D.rho, D.gam, D.vd_damping, nullptr, &zero, tw[0], tw[1],
                               tw[2], tw[3], tw[4], tw[5], tw[6], tw[7], tw[8], tw[9], tw[10], tw[11], m[M_DIP],
                               m[M_DIU], m[M_DIV], m[M_DIX], m[M_DJP], m[M_DJU], m[M_DJV], m[M_DJX], m[M_RU],
                               m[M_RV], D.dkp, D.dkw));
    }
    // the eddy viscosity and the three predictors convert the same fields
    // (u, v, w, and p, rho, rhonp1, gam) and tables to FP32 once: none of
    // them changes from the eddy viscosity to the last predictor
    struct F32Scope {
        Ctx &c;
        explicit F32Scope(Ctx &cc) : c(cc)
        {
            c.next32 = 0;
            c.f32_cache.clear();
            c.f32_scope = true;
        }
        ~F32Scope()
        {
            c.f32_scope = false;
            c.f32_cache.clear();
        }
    };
    F32Scope f32s(c);
    RET(need({D.gam, D.sc1, D.sc1var, D.gamsc1, D.sc1dis}));
    RET(lester_subgrid(D.gam, D.gamsc1, D.u, D.v, D.w, D.sc1, D.rho, D.sc1var, D.sc1dis, D.vd_damping, m[M_DIP],
                       m[M_DIU], m[M_DJP], m[M_DJV], D.dkp, D.dkw, m[M_HIJP], m[M_HJIP], m[M_HKIP], m[M_HKJP],
                       m[M_RP], nullptr, nullptr));
    RET(lester_set_gamsc1_bc(D.sc1, D.gamsc1, D.gamlam, m[M_DIU], m[M_DJV], D.dkp, m[M_RP]));
    RET(need({D.hn_sc1}));  // set_sc1 does not read p
    RET(lester_set_sc1(D.u, D.v, D.w, D.p, D.sc1, D.rho, D.gamsc1, D.gamlam, D.hn_sc1, m[M_DIP], m[M_DIU],
                       m[M_RDIV], m[M_DJP], m[M_DJV], m[M_RDJU], m[M_DIDJP], m[M_RDIDJP], m[M_HKIP], m[M_HKJP],
                       m[M_HKIU], m[M_HKJV], m[M_RP], D.dkp, D.dkw, nullptr, nullptr));
    RET(lester_set_sc1_bc(D.sc1));
    RET(lester_set_sc1var(D.u, D.v, D.w, D.sc1, D.rho, D.sc1var, D.sc1dis, m[M_DIP], m[M_DJP], D.dkp, D.dkw,
                          m[M_RP], nullptr, nullptr));
    RET(need({D.temperature}));  // rhonp1: written whole by search_lib, not copied in
    RET(lester_search_lib(D.sc1, D.sc1var, D.rhonp1, D.temperature, nullptr, nullptr, istep, &k.alpha, D.rho,
                          &k.rholo, &k.rhohi));
    RET(lester_set_sc1_bc(D.sc1));
    RET(lester_set_sc1_bc(D.rhonp1));
    RET(lester_set_sc1_bc(D.temperature));
    // final for this step: the eddy viscosities, the wall damping, the
    // scalar's right-hand side, variance and dissipation, the temperature
    RET(put({D.gam, D.gamsc1, D.gamlam, D.vd_damping, D.sc1dis, D.sc1var, D.temperature, D.hn_sc1}));
    // rhonp1 is final too, and swap_rhos ends the step with rho = rhonp1:
    // the caller's rho is copied back from rhonp1 now
    RET(put({D.rhonp1}));
    if (c.xfer) RET(c.xfer->put_as(D.rhonp1, D.rho));
    RET(need({D.p, D.hn_u}));
    {
        RET(lester_set_uv_int(&iU, D.u, D.v, D.w, D.p, D.rho, D.rhonp1, D.gam, D.u_int, D.hn_u, m[M_DIP], m[M_DIU],
                              m[M_DIX], m[M_RDIX], m[M_DJP], m[M_DJU], m[M_DJV], m[M_DJX], m[M_RDJP], m[M_RDJU],
                              m[M_DIDJP], m[M_DIDJU], m[M_RDIDJU], m[M_HIJP], m[M_HIJU], m[M_HJIU], m[M_HKIU],
                              m[M_HKJU], m[M_RP], m[M_RU], D.dkp, D.dkw, tw[0], tw[1], tw[2], tw[3], nullptr,
                              nullptr));
        RET(exitbc(1, 1));
        RET(need({D.hn_v}));
        // ---- ivar = v (step.F:319-326: the v arrays in the u roles)
        RET(lester_set_uv_int(&iV, D.v, D.u, D.w, D.p, D.rho, D.rhonp1, D.gam, D.v_int, D.hn_v, m[M_DJP], m[M_DJV],
                              m[M_DJX], m[M_RDJX], m[M_DIP], m[M_DIV], m[M_DIU], m[M_DIX], m[M_RDIP], m[M_RDIV],
                              m[M_DIDJP], m[M_DJDIV], m[M_RDJDIV], m[M_HJIP], m[M_HJIV], m[M_HIJV], m[M_HKJV],
                              m[M_HKIV], m[M_RP], m[M_RV], D.dkp, D.dkw, tw[4], tw[5], tw[6], tw[7], nullptr,
                              nullptr));
        RET(exitbc(1, 2));
        RET(need({D.hn_w}));
        // ---- ivar = w
        RET(lester_set_w_int(D.u, D.v, D.w, D.p, D.rho, D.rhonp1, D.gam, D.w_int, D.hn_w, m[M_DIP], m[M_DIU],
                             m[M_RDIV], m[M_DJP], m[M_DJV], m[M_RDJU], m[M_DIDJP], m[M_RDIDJP], m[M_HKIP], m[M_HKJP],
                             m[M_HKIU], m[M_HKJV], m[M_RP], m[M_RU], D.dkp, D.dkw, tw[10], tw[11], tw[8], tw[9],
                             nullptr, nullptr));
        RET(exitbc(1, 3));
        // the wall arrays (set_virt_bc, then the predictors) are final; the
        // predictors' right-hand sides too unless an outflow side updates them
        // after the projection (conv_exitbc task 2)
        for (int q = 0; q < 12; q++) RET(put({tw[q]}));
        if (!has_convective(c)) RET(put({D.hn_u, D.hn_v, D.hn_w}));
    }
    // ---- ivar = p
    if (*istep == 1)
        RET(lester_coeff_p(m[M_DIU], m[M_DJV], m[M_RDIV], m[M_RDJU], m[M_DIDJP], m[M_RP], D.dkp, D.dkw, D.ap, D.aw,
                           D.ae, D.as, D.an, D.al, D.ar));
    RET(lester_sour_p(m[M_DIU], m[M_DJV], m[M_RDIV], m[M_RDJU], m[M_DIDJP], D.dkp, m[M_RDIDJP], D.dkw, D.u_int,
                      D.v_int, D.w_int, D.rho, D.rhonp1, D.drhonp1dt, D.s, D.srhot, D.srhoux, nullptr, nullptr));
    return 0;
}

// step.F:420-454 after the Poisson solve: extrap_p, p_ref_subtract, the
// projection, slip sides, outflow updates, the density rotation
static int step_post(Ctx &c, lester_fields &D, const int *istep)
{
    double *const *m = D.metric;
    const double *mx[12] = {m[M_DIP], m[M_DIU], m[M_DIX], m[M_DJP], m[M_DJV], m[M_DJX],
                            m[M_RDIV], m[M_RDJU], m[M_DIDJP], m[M_RP], m[M_RU], m[M_RV]};
    // conv_exitbc(task, iva) of step.F:344 and 435
    auto exitbc = [&](int task, int iva) {
        return exit_task(c, task, iva, D.rho, D.rhonp1, D.u, D.v, D.w, D.u_int, D.v_int, D.w_int, D.hn_u, D.hn_v,
                         D.hn_w, mx, D.dkp, D.dkw, m[M_RDIDJP]);
    };
    const int iU = 1, iV = 2, iW = 3;
    RET(lester_extrap_p(D.p, nullptr, nullptr));
    RET(lester_p_ref_subtract(D.p));
    RET(lester_uvw_adv(&iU, m[M_DIU], m[M_RP], D.dkw, D.u, D.u_int, D.rhonp1, D.p, nullptr, nullptr, istep));
    RET(lester_uvw_adv(&iV, m[M_DJV], m[M_RP], D.dkw, D.v, D.v_int, D.rhonp1, D.p, nullptr, nullptr, istep));
    RET(lester_uvw_adv(&iW, m[M_DIU], m[M_RP], D.dkw, D.w, D.w_int, D.rhonp1, D.p, nullptr, nullptr, istep));
    RET(lester_slipbc(nullptr, nullptr, nullptr, m[M_DIP], m[M_DIU], m[M_DJP], m[M_DJV], D.dkp, D.u, D.v, D.v_int,
                      D.w, D.sc1, D.rho, D.p, istep));
    for (int iva = 1; iva <= 3; iva++) RET(exitbc(2, iva));
    RET(lester_swap_rhos(D.rho, D.rhonp1, D.rhonm1));
    return 0;
}

// ---- the whole step as one CUDA graph (ctrl.step_graph) -----------------
// Capture: step_pre, the fast solve as a device-controlled loop (a WHILE
// node, fast_solve_graph), then step_post inside an IF node that runs when
// the solve converged or used its cycles -- the cases in which the step
// as launched carries on.  The loop state is copied to pinned memory at
// the end; the step counter of the predictors' running means is copied in
// at the start.  Nothing runs while capturing, so a capture that fails
// leaves the state as it was and the step runs as launched.
static int p_guess(Ctx &c, lester_fields &D, const int *istep);

static int step_capture(Ctx &c, lester_fields &D, const int *istep)
{
    if (c.sg.exec) cudaGraphExecDestroy(c.sg.exec);
    c.sg.exec = nullptr;
    // step counters of a replay: [0] iststep (the predictors' running
    // means), [1] the caller's istep (the inlet perturbations)
    if (!c.h_step) LES_CUDA(cudaMallocHost(&c.h_step, 2 * sizeof(int)));
    if (!c.h_loop) LES_CUDA(cudaMallocHost(&c.h_loop, 8 * sizeof(double)));
    if (!c.d_step) LES_CUDA(cudaMalloc(&c.d_step, 2 * sizeof(int)));
    if (!c.d_loop) LES_CUDA(cudaMalloc(&c.d_loop, 8 * sizeof(double)));
    if (!c.cap_stream) LES_CUDA(cudaStreamCreateWithFlags(&c.cap_stream, cudaStreamNonBlocking));
    if (!c.graph_stream) LES_CUDA(cudaStreamCreateWithFlags(&c.graph_stream, cudaStreamNonBlocking));
    LES_CUDA(cudaStreamSynchronize(c.stream));
    cudaGetLastError();
    const long l0 = launch_count();
    // captured on a stream of our own; the graph is launched on c.stream
    const cudaStream_t user = c.stream;
    c.stream = c.graph_stream;
    if (cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        c.stream = user;
        cudaGetLastError();
        return set_err(LES_ERR_CUDA, "step graph: cannot begin the capture");
    }
    c.capturing = true;
    int r = 0;
    if (cudaMemcpyAsync(c.d_step, c.h_step, 2 * sizeof(int), cudaMemcpyHostToDevice, c.stream) != cudaSuccess ||
        cudaMemsetAsync(c.d_loop, 0, 8 * sizeof(double), c.stream) != cudaSuccess)
        r = set_err(LES_ERR_CUDA, "step graph: status copies");
    if (!r && c.xfer) r = c.xfer->issue_in();  // host inputs: copy nodes
    if (!r) r = step_pre(c, D, istep);
    if (!r) r = p_guess(c, D, istep);
    if (!r) {
        c.want_norms = false;
        r = lester_lmg_solve(D.ap, D.aw, D.ae, D.as, D.an, D.al, D.ar, D.p, D.s, D.res, nullptr, nullptr);
        c.want_norms = true;
    }
    if (!r) {
        cudaGraph_t body;
        cudaStream_t saved;
        r = graph_add_conditional(c, c.sg_post, cudaGraphCondTypeIf, &body);
        if (!r) r = graph_begin_body(c, body, &saved);
        if (!r) {
            r = step_post(c, D, istep);
            const int r2 = graph_end_body(c, saved);
            if (!r) r = r2;
        }
    }
    if (!r && cudaMemcpyAsync(c.h_loop, c.d_loop, 8 * sizeof(double), cudaMemcpyDeviceToHost, c.stream) != cudaSuccess)
        r = set_err(LES_ERR_CUDA, "step graph: status copy");
    // host outputs not copied during the step, then both copy branches
    // rejoin the capture's stream
    if (!r && c.xfer) r = c.xfer->put_rest();
    if (!r && c.xfer) r = c.xfer->join();
    c.capturing = false;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c.stream, &g);
    c.stream = user;
    const long captured = launch_count() - l0;
    count_launch(-captured);  // captured, not launched
    if (r || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return r ? r : set_err(LES_ERR_CUDA, "step graph capture: %s", cudaGetErrorString(e));
    }
    const cudaError_t ei = cudaGraphInstantiate(&c.sg.exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        cudaGetLastError();
        c.sg.exec = nullptr;
        return set_err(LES_ERR_CUDA, "step graph instantiate: %s", cudaGetErrorString(ei));
    }
    c.sg.launches = captured;
    return 0;
}

// The step by its graph.  *done is false when it is not eligible or
// cannot be captured (the caller runs it as launched); otherwise the return
// value is the step's.
static int step_graph_run(Ctx &c, lester_fields &D, const int *istep);

static int step_graph(Ctx &c, lester_fields &D, const lester_fields &H, const int *istep, bool *done)
{
    *done = false;
    const int ps = c.c.psolve;
    if (*istep == 1 || (ps != LES_PSOLVE_FP64 && ps != LES_PSOLVE_MIXED) || c.prof) return 0;
    const int prec = ps == LES_PSOLVE_MIXED ? 32 : 64;
    if (c.c.autotune && !c.tuned[prec == 32 ? 1 : 0].done) return 0;
    // the coefficients converted by an earlier solve of this precision
    const double *coef[7] = {D.ap, D.aw, D.ae, D.as, D.an, D.al, D.ar};
    bool ready = c.coef_prec == prec && c.coef_gen_seen == c.coef_gen;
    for (int q = 0; q < 7; q++) ready = ready && c.coef_key[q] == coef[q];
    if (!ready || (c.c.krylov == 1 && !c.d_fr) || (c.singular && !c.d_bmean)) return 0;
    const bool same = !memcmp(&c.sg.key, &D, sizeof D) && !memcmp(&c.sg.hkey, &H, sizeof H) &&
                      !memcmp(&c.sg.ctrl, &c.c, sizeof c.c) && c.sg.coef_gen == c.coef_gen;
    if (same && c.sg.failed) return 0;
    if (!same || !c.sg.exec) {
        c.sg.key = D;
        c.sg.hkey = H;
        c.sg.coef_gen = c.coef_gen;
        c.sg.failed = step_capture(c, D, istep) != 0;
        c.sg.ctrl = c.c;  // as the capture left it (with any autotuned settings)
        if (c.sg.failed) {
            c.sg.why = g_err;
            g_err.clear();
            return 0;
        }
    }
    *done = true;
    if (c.xfer) c.xfer->in_graph();  // its copies are the graph's
    return step_graph_run(c, D, istep);
}

static int step_graph_run(Ctx &c, lester_fields &D, const int *istep)
{
    c.h_step[0] = c.iststep;
    c.h_step[1] = *istep;
    LES_CUDA(cudaGraphLaunch(c.sg.exec, c.stream));
    c.sg.replays++;
    LES_CUDA(cudaStreamSynchronize(c.stream));
    const double *h = c.h_loop;
    const int status = (int)h[4], cycles = (int)h[3];
    count_launch(c.sg.launches + (long)(cycles - 1) * c.sg.body_launches);
    c.last_cycles = cycles;
    c.last_relres = h[1];
    c.last_solve_ms = -1;  // not timed inside the graph
    {
        const double rn = 1.0 / c.lv[1].npts_all, bn = std::sqrt(h[0] * rn);
        c.last_norms[0] = h[1] * bn;  // rnorm from ||r|| / ||b|| and ||b||^2
        c.last_norms[1] = bn;
        c.last_norms[2] = c.last_norms[3] = 0.;
    }
    if (h[6] != 0) return set_err(LES_ERR_TIMEOUT, "set_sc1: grid barrier of the scalar sweep timed out");
    if (status == 4) return set_err(LES_ERR_NONFINITE, "non-finite residual after %d cycles", cycles);
    if (status == 3 || status == 5) {
        // the host loop takes over: flexible CG from the current p with the
        // cycles left, then the rest of the step
        const int maxit = c.c.max_outer > 0 ? c.c.max_outer : 100;
        c.sg.handovers++;
        c.force_krylov = true;
        c.cycle_budget = std::max(0, maxit - cycles);
        c.want_norms = false;
        int rs = lester_lmg_solve(D.ap, D.aw, D.ae, D.as, D.an, D.al, D.ar, D.p, D.s, D.res, nullptr, nullptr);
        c.want_norms = true;
        c.last_cycles += cycles;
        if (rs && rs != LES_ERR_NOT_CONVERGED) return rs;
        RET(step_post(c, D, istep));
        if (c.xfer) RET(c.xfer->copy_out_all());  // the graph copied the outputs before this
        c.iststep += 1;
        return rs;
    }
    c.iststep += 1;
    if (status == 2)
        return set_err(LES_ERR_NOT_CONVERGED, "relative residual %.3e after %d cycles", h[1], cycles);
    return 0;
}

static int step_body(Ctx &c, lester_fields *F, const int *istep);

// The initial pressure of a fast solve with ctrl.p_guess 1: 2 p(n) - p(n-1)
// once the previous step's solve started from a solution (k_p_guess); the
// arrays are allocated on a launched step, never while capturing.
static int p_guess(Ctx &c, lester_fields &D, const int *istep)
{
    const int ps = c.c.psolve;
    if (c.c.p_guess != 1 || (ps != LES_PSOLVE_FP64 && ps != LES_PSOLVE_MIXED)) return 0;
    if (!c.p_prev) {
        if (c.capturing) return 0;
        if (cudaMalloc(&c.p_prev, sizeof(double) * (size_t)c.tot_sg3) != cudaSuccess ||
            cudaMalloc(&c.d_pguess, sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(c.p_prev);
            c.p_prev = nullptr;
            return set_err(LES_ERR_NOMEM, "p_guess: previous pressure");
        }
        LES_CUDA(cudaMemsetAsync(c.d_pguess, 0xff, sizeof(int), c.stream));  // -1: none
    }
    launch_p_guess(D.p, c.p_prev, c.tot_sg3, *istep, c.capturing ? c.d_step + 1 : nullptr, c.d_pguess, c.stream);
    return 0;
}

// the step, and its JSON line when a step log is open (lester_gpu_step_log)
int lester_step(lester_fields *F, const int *istep)
{
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    if (!c.step_log) return step_body(c, F, istep);
    const long h0 = c.h2d_bytes, d0 = c.d2h_bytes, rep0 = c.sg.replays;
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = step_body(c, F, istep);
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    // the discrete divergence of the projected velocity is the pressure
    // equation's residual: resid_rms (rnorm of code/norms.F) measures it
    std::fprintf(c.step_log,
                 "{\"istep\": %d, \"rc\": %d, \"ms\": %.4f, \"vcycles\": %d, \"relres\": %.6e, "
                 "\"resid_rms\": %.6e, \"rhs_rms\": %.6e, \"graph\": %s, \"h2d_bytes\": %ld, "
                 "\"d2h_bytes\": %ld}\n",
                 istep ? *istep : -1, rc, ms, c.last_cycles, c.last_relres, c.last_norms[0], c.last_norms[1],
                 c.sg.replays != rep0 ? "true" : "false", c.h2d_bytes - h0, c.d2h_bytes - d0);
    std::fflush(c.step_log);
    return rc;
}

int lester_gpu_step_log(const char *path)
{
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    if (c.step_log) std::fclose(c.step_log);
    c.step_log = nullptr;
    if (!path || !*path) return 0;
    c.step_log = std::fopen(path, "a");
    if (!c.step_log) return set_err(LES_ERR_ARG, "step log: cannot open %s", path);
    return 0;
}

static int step_body(Ctx &c, lester_fields *F, const int *istep)
{
    if (!F || !istep) return set_err(LES_ERR_ARG, "null fields / istep");
    int r0;
    if ((r0 = ensure_sides(c))) return r0;
    if (has_inlet(c) && (!c.d_uprof || !c.d_vprof))
        return set_err(LES_ERR_ARG, "inlet blocks set without profiles (lester_gpu_set_inlet)");
    // Host arrays are mirrored once for the step.  What crosses: the
    // fields a step reads before it writes them (the carried state) are
    // copied in, the fields the caller reads afterwards (the state and the
    // outputs of the eddy viscosity, scalar and density) are copied back;
    // only level 1 of p crosses; the predictor's and the solver's work
    // arrays (u_int, v_int, w_int, s, res, the sour_p diagnostics)
    // stay in library-held device arrays; the metrics only come in; the
    // pressure coefficients, which coeff_p writes at istep 1 and no later
    // step changes (as in the reference), cross back at istep 1 and are
    // kept on the device for the host arrays they mirror.  Inputs are
    // mapped in the order the step first reads them, the order of their
    // copies.
    Staging st(&c, __func__);
    st.defer();
    lester_fields D = *F;
    long n3 = c.tot_sg3, nm = c.tot3;
    int r;
    for (int q = 0; q < 35; q++) {
        if (!D.metric[q]) return set_err(LES_ERR_ARG, "metric %d missing", q);
        RET(st.in(D.metric[q], c.tot2, (const double **)&D.metric[q]));
    }
    RET(st.in(D.dkp, c.tot1k, (const double **)&D.dkp));
    RET(st.in(D.dkw, c.tot1k, (const double **)&D.dkw));
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
    if (!D.p || !D.s || !D.res) return set_err(LES_ERR_ARG, "p, s, res and the coefficient arrays are required");
    enum { IO, OUT, WORK, P };
    struct F3 {
        double **pp;
        int role;
    } f3[] = {{&D.u, IO},         {&D.rho, IO},         {&D.vd_damping, IO}, {&D.v, IO},
              {&D.w, IO},         {&D.gam, IO},         {&D.sc1, IO},        {&D.sc1var, IO},
              {&D.gamsc1, IO},    {&D.sc1dis, IO},      {&D.gamlam, OUT},    {&D.hn_sc1, IO},
              {&D.rhonp1, OUT},   {&D.temperature, IO}, {&D.p, P},           {&D.hn_u, IO},
              {&D.hn_v, IO},      {&D.hn_w, IO},        {&D.rhonm1, OUT},    {&D.u_int, WORK},
              {&D.v_int, WORK},   {&D.w_int, WORK},     {&D.drhonp1dt, WORK}, {&D.srhot, WORK},
              {&D.srhoux, WORK}};
    int nscr = 0;
    // a library-held device array of n elements (zeroed at first use)
    auto scratch = [&](long n, double **pp) -> int {
        if ((int)c.scratch.size() <= nscr) {
            double *d = nullptr;
            if (cudaMalloc(&d, sizeof(double) * nm) != cudaSuccess) {
                cudaGetLastError();
                return set_err(LES_ERR_NOMEM, "step scratch allocation failed");
            }
            cudaMemsetAsync(d, 0, sizeof(double) * nm, c.stream);
            c.scratch.push_back(d);
        }
        (void)n;
        *pp = c.scratch[nscr++];
        return 0;
    };
    auto is_host = [](const double *p) {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
            cudaGetLastError();
            return true;
        }
        return at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged;
    };
    for (const F3 &f : f3) {
        double **pp = f.pp;
        if (f.role == P) RET(st.io_part(D.p, nm, n3, &D.p));  // level 1 crosses; the coarser levels are solver work
        else if (!*pp || (f.role == WORK && is_host(*pp))) RET(scratch(n3, pp));  // NULL, or a host work array
        else if (f.role == OUT) RET(st.out(*pp, n3, pp));
        else RET(st.io(*pp, n3, pp));
    }
    if (is_host(D.s)) RET(scratch(nm, &D.s));
    if (is_host(D.res)) RET(scratch(nm, &D.res));
    double **fc[] = {&D.ap, &D.aw, &D.ae, &D.as, &D.an, &D.al, &D.ar};
    for (int q = 0; q < 7; q++) {
        double **pp = fc[q];
        if (!*pp) return set_err(LES_ERR_ARG, "p, s, res and the coefficient arrays are required");
        if (!is_host(*pp)) continue;
        const double *h = *pp;
        if (!c.coef_mirror[q]) {
            if (cudaMalloc(&c.coef_mirror[q], sizeof(double) * nm) != cudaSuccess) {
                cudaGetLastError();
                c.coef_mirror[q] = nullptr;
                return set_err(LES_ERR_NOMEM, "coefficient mirror allocation failed");
            }
            c.coef_host[q] = nullptr;
        }
        if (*istep == 1) {
            // written by coeff_p in this step into the mirror, copied back
            // to the host array by finish()
            st.out_from(const_cast<double *>(h), c.coef_mirror[q], nm);
            c.coef_host[q] = h;
            *pp = c.coef_mirror[q];
        } else if (c.coef_host[q] != h) {
            LES_CUDA(cudaMemcpyAsync(c.coef_mirror[q], h, sizeof(double) * nm, cudaMemcpyHostToDevice, c.stream));
            c.h2d_bytes += nm * (long)sizeof(double);
            c.coef_host[q] = h;
            *pp = c.coef_mirror[q];
        } else {
            *pp = c.coef_mirror[q];
        }
    }
    // the deferred copies of this call (step_pre's waits and early puts)
    struct XferScope {
        Ctx &c;
        XferScope(Ctx &cc, Staging *s) : c(cc) { c.xfer = s; }
        ~XferScope() { c.xfer = nullptr; }
    } xscope(c, st.any_host() ? &st : nullptr);
    if (c.c.step_graph && !st.pageable()) {
        // device pointers are stable from call to call (staging buffers by
        // call order, library arrays): the graph keyed on them and on the
        // host arrays it copies replays, the host copies as its nodes
        bool done = false;
        const int rg = step_graph(c, D, *F, istep, &done);
        if (done) {
            if (rg && rg != LES_ERR_NOT_CONVERGED) return rg;
            const int rf = st.finish();
            return rf ? rf : rg;
        }
        st.clear_marks();
    }
    RET(st.issue_in());
    RET(step_pre(c, D, istep));
    RET(p_guess(c, D, istep));
    c.want_norms = false;
    int rs = lester_lmg_solve(D.ap, D.aw, D.ae, D.as, D.an, D.al, D.ar, D.p, D.s, D.res, nullptr, nullptr);
    c.want_norms = true;
    // the reference carries on after nummgits cycles whatever the residual;
    // a fast solver that stops short reports it and the step continues
    if (rs && rs != LES_ERR_NOT_CONVERGED) return rs;
    RET(step_post(c, D, istep));
    c.iststep += 1;  // code/step.F:181, ready for the next step
    r = st.finish();
    if (r) return r;
    return rs;
}

// steps run by replaying the whole-step graph since lester_gpu_init, and
// whether the graph for the current fields failed to capture
int lester_gpu_step_graph_info(long *replays, long *handovers, int *failed, char *why, int why_len)
{
    LES_NEED_CTX();
    if (replays) *replays = g_ctx->sg.replays;
    if (handovers) *handovers = g_ctx->sg.handovers;
    if (failed) *failed = g_ctx->sg.failed ? 1 : 0;
    if (why && why_len > 0) {
        snprintf(why, (size_t)why_len, "%s", g_ctx->sg.failed ? g_ctx->sg.why.c_str() : "");
    }
    return 0;
}

} // extern "C"
