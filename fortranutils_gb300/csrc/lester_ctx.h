// lester_ctx.h -- host-side state of the library (what the reference keeps
// in COMMON blocks) and helpers shared by the host translation units.
#pragma once
#include <cstdio>
#include <cuda_runtime.h>
#include <string>
#include <vector>
#include "../../include/lester_gpu.h"
#include "k_common.cuh"
#include "phys_args.h"
#include "kernels.h"

namespace les {

struct LevelGeom {
    int n[LES_MAXBL + 1][3];
    int mult[LES_MAXBL + 1][3];
    long off3[LES_MAXBL + 1], off2[LES_MAXBL + 1], off1k[LES_MAXBL + 1];
    long offxy[LES_MAXBL + 1], offz[LES_MAXBL + 1];
    long maxcell, maxjk, maxhalf, maxfine, maxik, maxface, maxij, maxk;
    int maxn[3];  // the most points of a block along i, j, k (ghosts included)
    long start3, len3;     // contiguous range of this level in a 3-D mg field
    double npts_all;       // interior points, pressure loop bounds (set_loop_bound.F:364)
    BlkDev *d_blk = nullptr;
    FaceDev *d_face = nullptr;
    PushDev *d_push = nullptr;  // 6 per block: ghost mirrors of the interior planes
    LevGeo geo;                 // the level as a kernel parameter (geo_ok: at most kGeoBlk blocks)
    ZMap zint, zpro;            // (block, plane) maps: interior planes; planes 1 .. n[2] - 1
    int2 *d_zmaps = nullptr;    // both maps in one allocation
    bool geo_ok = false;
    // red-black sweeps may push: on every face the point a ghost mirrors and
    // the point that reads that ghost have different colours
    bool rb_push = true;
    int nface = 0;
    long worklen = 0;
    void *d_metblk = nullptr;
    void *d_metface[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int nmetface[6] = {0, 0, 0, 0, 0, 0};
    long maxmetlen = 0;
};

// One defect-correction iteration of a fast solver (V-cycle, update, halo,
// FP64 residual, read-back of two sums) captured as a CUDA graph.
struct Tuned {
    bool done = false;
    int threads = 256, sweeps = 3, tail = 4096, line = 0;
    int seen = 0;  // solves before tuning
    double omega = 1.5;
};

struct CycleGraph {
    cudaGraphExec_t exec = nullptr;
    const void *f = nullptr, *b = nullptr;
    int sweeps = 0, coarse = 0;
    double omega = 0;
    bool singular = false;
    bool mf = false;
    int tail = 0;
    int krylov = 0;
    int threads = 0;                // red-black CTA size
    int line = 0;                   // y-line relaxation
    int direct = 0;                 // points of the bottom level's direct solve (0: smoothed)
    int dfsep = 0;                  // Ctx::df_sep
    int tile = 0;                   // ctrl.rb_tile
    long launches = 0;              // kernels per replay
    std::vector<cudaEvent_t> ev;    // pairs around the level-1 smoother launches
};

// device buffers of the fast solvers, precision T
template <typename T> struct FastSet {
    T *E = nullptr, *N = nullptr, *R = nullptr, *D = nullptr, *x = nullptr, *b = nullptr;
    T *cp = nullptr, *dp = nullptr;  // y-line Thomas scratch (all levels), at first use
    MfTab<T> tab;       // separable factors (FP32 solver)
    bool mf = false;    // tab checked against every coefficient: used
    T *x2 = nullptr;    // the other buffer of the shared-memory red-black sweeps (k_rb_tile)
    T *cmt = nullptr;   // dense inverse of the bottom level (CoarseDirect), kDirectMax^2
    int cn = 0;         // its points (0: the bottom level is smoothed)
    int clev = 0;       // its level
};

struct Ctx {
    lester_geom g;
    lester_ctrl c;
    int nummgl = 0;
    LevelGeom lv[LES_MAXMGL + 1];
    long tot3 = 0, tot_sg3 = 0, tot2 = 0, tot1k = 0, totxy = 0, totz = 0, totki = 0, totjk = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int jumble = 0;
    // scratch
    double *d_work = nullptr;       // swap pack buffer
    double *d_partial = nullptr;    // reduction partials
    long npartial = 0;
    double *d_small = nullptr;      // small results (norms, p_ref)
    double *h_small = nullptr;      // pinned mirror
    double *d_nrm3 = nullptr;       // per-point SOR norm terms (reference smoother)
    double *d_metbuf = nullptr;
    long metslot = 0;
    long metmaxf = 0;
    int *d_flag = nullptr;
    // fast solvers
    FastSet<float> f32;
    FastSet<double> f64;
    double *E64 = nullptr, *N64 = nullptr, *R64 = nullptr, *P64 = nullptr;
    // the mixed solver's outer iteration in double-float (k_dfloat.cu): the
    // level-1 coefficients, p and b - shift as FP32 pairs
    double *p_prev = nullptr;  // level-1 p at the start of the previous step's fast solve (ctrl.p_guess)
    int *d_pguess = nullptr;   // the istep p_prev was taken at (device; -1: none)
    std::FILE *step_log = nullptr;  // lester_gpu_step_log's file (one JSON line per lester_step)
    float2 *df_E = nullptr, *df_N = nullptr, *df_R = nullptr, *df_P = nullptr, *df_p = nullptr, *df_b = nullptr;
    // separable double-float factors of the level-1 couplings; df_sep: 0
    // not in use (the arrays above), 1 couplings from the factors and the
    // diagonal from df_P, 2 the diagonal as the couplings' sum too
    DfTab df_tab;
    int df_sep = 0;
    double *d_fr = nullptr, *d_fp = nullptr, *d_fq = nullptr;  // flexible CG: r, p, q (level 1)
    // convective outflow / fixed inflow sides (lester_outflow.cu)
    bool sides_built = false;
    std::vector<SideJob> sides;     // (block, side) order
    SideJob *d_sides = nullptr;
    double *d_exit = nullptr;       // EX_N SAVEd values
    double *d_sideout = nullptr;    // 3 sums per side
    int inlet[4] = {0, 0, 0, 0};    // inlet blocks (1-based; 0 none)
    double *d_uprof = nullptr, *d_vprof = nullptr;
    int nprof = 0;
    unsigned long long inlet_seed = 0;
    int no_sam = 1;                 // statistics: samples so far (COMMON no_sam)
    int ncomp = 1;                  // connected components of the block graph
    int rb_threads = 256;           // red-black launch shape (autotuned)
    Tuned tuned[2];                 // autotuned solver settings [FP64, mixed]
    double *d_bmean = nullptr;      // per block: interior mean of b over its component
    const void *coef_key[7] = {0, 0, 0, 0, 0, 0, 0};
    long coef_gen_seen = -1;
    int coef_prec = -1;
    bool singular = true;   // pure Neumann/periodic operator (constant null vector)
    long coef_gen = 0;
    // staging buffers for host arguments
    std::vector<void *> stage_buf;
    std::vector<size_t> stage_cap;
    // copy streams and events of lester_step's deferred host copies
    cudaStream_t xs_in = nullptr, xs_out = nullptr;
    std::vector<cudaEvent_t> xev;
    class Staging *xfer = nullptr;  // the running lester_step's host copies
    // kernel timing inside a timed region (lester_gpu_prof): CUDA events
    // around every launch of the timed kernels (LES_PROF_*): pairs in
    // ev_pool, the kernel of pair q in ev_tag[q]
    bool prof = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<int> ev_tag;
    size_t ev_used = 0;
    long prof_launches[2] = {0, 0};
    double prof_ms_acc[2] = {0, 0};
    // graphs of the fast solvers: [FP64, mixed][defect correction, flexible CG]
    CycleGraph cg[2][3];  // [FP64, mixed][defect correction, flexible CG, double-float defect correction]
    cudaStream_t cap_stream = nullptr;
    std::vector<cudaEvent_t> *cap_ev = nullptr;  // set while capturing
    // bytes copied between host and device by staged (host-array) calls
    long h2d_bytes = 0, d2h_bytes = 0;
    // predictor / scalar tables (lester_phys_host.cu)
    long *d_offki = nullptr, *d_offjk = nullptr;
    int *d_link = nullptr;
    double *d_grad = nullptr;
    long gstride = 0, maxfacecell = 0, tot2_l1 = 0;
    int gm = 0;
    int iststep = 2;  // step.F:180 increments it once before the first step
    int init_vdd[LES_MAXBL][6] = {};
    std::vector<double *> scratch;  // step fields the caller left NULL, or host work arrays lester_step keeps on the device
    // lester_step with host arrays: device mirrors of the pressure
    // coefficients (written at istep 1 by coeff_p, then only read), keyed
    // by the host array they mirror
    double *coef_mirror[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    const double *coef_host[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // last solve statistics
    double last_norms[4] = {0, 0, 0, 0};
    int last_cycles = 0;
    double last_relres = 0;
    double last_solve_ms = 0;              // device time of the last fast solve
    bool want_norms = true;  // fast solves end with the reference-style norms and residu
    double *d_tabpool = nullptr;  // tables of the fast physics kernels
    // persistent scalar sweep: per plane, cumulative point counts over the
    // (block, k) slices; the slices; the grid barrier
    int *d_wcum = nullptr;
    int2 *d_wslice = nullptr;
    int nslice = 0;
    WaveSync *d_wave = nullptr;
    // tiled scalar sweep (k_sweep.cu): per-block skew geometry, the tiles in
    // ticket order, ticket + error, skewed copies per storage type (FP64 for
    // the FP64 builds, FP32 for phys32)
    struct SweepState {
        SkewBlk *d_sb = nullptr;
        int maxn[3] = {0, 0, 0};
        long tot3 = 0, tot2 = 0;      // skewed elements per 3-D field / 2-D table
        int *d_sync = nullptr;        // ticket, error
        void *d_sk[2] = {nullptr, nullptr};  // [FP64, FP32]: 8 fields, the new values, 10 tables
        // per physics build [exact, fast, FP32]: rows per tile follow the
        // build's shared-memory ring
        SweepTile *d_tiles[3] = {nullptr, nullptr, nullptr};
        int ntile[3] = {0, 0, 0};
        int sw[3] = {0, 0, 0};        // ring row width (elements)
        int nthr[3] = {0, 0, 0};      // threads per CTA: row warps + the producer warp
        int maxctas[3] = {0, 0, 0};   // resident CTAs; -1 none
        void *d_tmaps[3] = {nullptr, nullptr, nullptr};  // TMA tensor maps over d_sk (k_sweep.cu)
    } sw;
    VLev *d_vlev = nullptr;  // per-level descriptors (index = level) for k_vtail
    bool vtail_smem = false; // k_vtail may stage its slice in shared memory
    bool rb_tile_ok = false; // k_rb_tile's shared memory granted
    int rb_tile_mask = 0;    // levels (bit lev) the last cycle smoothed with k_rb_tile
    const double *fb[3] = {nullptr, nullptr, nullptr};  // body force u, v, w (device)
    long tabcap = 0, tab_next = 0;
    float *d_pool32 = nullptr;      // FP32 copies of the tables (phys32), reset per call
    long cap32 = 0, next32 = 0;
    // lester_step's three predictor calls share their FP32 copies of the
    // caller's arrays (none of them changes between the calls): while
    // f32_scope is set the pool is not rewound and a copy is reused for the
    // same array and length (not for the per-call tables of d_tabpool)
    bool f32_scope = false;
    struct F32Copy {
        const double *src;
        long len;
        float *dst;
    };
    std::vector<F32Copy> f32_cache;
    cudaEvent_t ev_solve[2] = {nullptr, nullptr};
    // whole-step graph (ctrl.step_graph, lester_step.cu)
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        lester_fields key{};  // the fields it was captured with (device)
        lester_fields hkey{}; // and as the caller passed them (host copies)
        lester_ctrl ctrl{};   // and the controls
        long coef_gen = -1;
        long launches = 0;    // kernels captured (the cycle loop's body once)
        long body_launches = 0;  // kernels of one cycle
        bool kry = false;     // its cycles are flexible CG
        bool failed = false;  // capture failed for this key: run as launched
        long replays = 0;     // steps run by replaying it
        long handovers = 0;   // of those, solves the host loop finished
        std::string why;      // the capture failure's message
    } sg;
    bool capturing = false;     // lester_step is being captured
    cudaStream_t graph_stream = nullptr;  // the capture's stream (the caller's may be the legacy one)
    cudaGraphConditionalHandle sg_post = 0;  // gate of the step after the solve
    int *d_step = nullptr;      // iststep of the replayed step (device copy)
    int *h_step = nullptr;      // its pinned host source
    double *d_loop = nullptr;   // cycle-loop state of the captured solve
    double *h_loop = nullptr;   // pinned copy of it, read after the step
    bool force_krylov = false;  // the next fast solve starts in flexible CG
    int cycle_budget = -1;      // and runs at most this many cycles (-1: max_outer)
};

// whole-step graph: conditional nodes inside the capture on c.stream
// (lester_host.cu)
int graph_cond_handle(Ctx &c, cudaGraphConditionalHandle *h);
int graph_add_conditional(Ctx &c, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, cudaGraph_t *body);
int graph_begin_body(Ctx &c, cudaGraph_t body, cudaStream_t *saved);
int graph_end_body(Ctx &c, cudaStream_t saved);

// phys32 (the les_f32 build): its read-only tables as FP32 copies, passed
// as pointers tagged in bit 0 (LdF in phys_variant.h reads them directly).
// phys32_tables replaces each *pp[t] (length len) by such a copy, refreshed
// on every call from a pool that phys32_reset rewinds (lester_phys_host.cu)
inline bool phys32_on(const Ctx &c) { return c.c.phys32 && !c.c.exact; }
void phys32_reset(Ctx &c);
int phys32_tables(Ctx &c, int n, const double **const *pp, long len);

extern Ctx *g_ctx;
extern std::string g_err;
int set_err(int code, const char *fmt, ...);
// fast physics kernels: reciprocals of n device tables of length len, and
// the split filter-width tables; slots are reused by the next call (same
// stream).  tab_reset starts a call.
void tab_reset(Ctx &c);
int recip_tabs(Ctx &c, int n, const double *const *src, long len, const double **out);
int delta_tabs(Ctx &c, const double *dip, const double *djp, const double *rp, const double *dkp,
               const double **d2, const double **d1);
int fast_sgs_tabs(Ctx &c, const double *dip, const double *djp, const double *rp, const double *dkp,
                  const double *dkw, SgsFast &F);
// the exact (bitwise) or fast build of the physics launchers
#define LES_PHYS(c, fn) ((c).c.exact ? les_exact::fn : (c).c.phys32 ? les_f32::fn : les_fast::fn)

// a pair of timing events for one launch of kernel `tag` (LES_PROF_*),
// used when c.prof is on and nothing is being captured
void prof_pair(Ctx &c, int tag, cudaEvent_t *e0, cudaEvent_t *e1);

// polls a bounded device wait makes before it gives up (ctrl.wait_limit)
inline long wait_polls(const Ctx &c) { return c.c.wait_limit > 0 ? (long)c.c.wait_limit : (1L << 24); }

#define LES_CUDA(call)                                                                             \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            cudaGetLastError(); /* reported here; not again by a later check */                    \
            return les::set_err(LES_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,          \
                                cudaGetErrorString(e_));                                           \
        }                                                                                          \
    } while (0)

// lester_outflow.cu: convective outflow / fixed inflow on device arrays;
// m[] = dip, diu, dix, djp, djv, djx, rdiv, rdju, didjp, rp, ru, rv
int ensure_sides(Ctx &c);
bool has_convective(const Ctx &c);
bool has_inlet(const Ctx &c);
int exit_task(Ctx &c, int task, int iva, const double *rho, const double *rhonp1, double *u, double *v,
              double *w, double *u_int, double *v_int, double *w_int, double *hu, double *hv, double *hw,
              const double *const *m, const double *dkp, const double *dkw, const double *rdidjp);
int inlet_task(Ctx &c, const double *uprof, const double *vprof, unsigned long long seed, int step, double *u,
               double *v, double *w, double *sc1, double *rho, double *u_int, double *v_int, double *w_int);

#define LES_NEED_CTX()                                                                             \
    do {                                                                                           \
        if (!les::g_ctx) return les::set_err(LES_ERR_NOT_INIT, "lester_gpu_init not called");      \
    } while (0)

// Maps the pointers of one entry-point call to device memory: device
// pointers pass through, host arrays are copied to library-owned device
// buffers and, for outputs, copied back by finish().
class Staging {
  public:
    // `who` names the entry point in error messages; an error already
    // pending on entry is reported as such rather than blamed on this call
    explicit Staging(Ctx *c, const char *who = "?") : c_(c), who_(who), pre_(cudaGetLastError()) {}
    ~Staging();
    // in: read only; io: read and written; out: written only (a host
    // array is not copied in); io_part: a device array of n elements of
    // which only the first ncopy cross to and from a host array
    int in(const double *user, long n, const double **dev);
    int io(double *user, long n, double **dev);
    int out(double *user, long n, double **dev);
    int io_part(double *user, long n, long ncopy, double **dev);
    // a host array written through a library-held device array `dev` of n
    // elements: copied back by finish()
    void out_from(double *user, double *dev, long n);
    int finish();  // copies outputs back and synchronises if anything was staged
    bool any_host() const { return any_host_; }
    bool pageable() const { return pageable_; }  // a host array is not page-locked

    // Deferred copies (lester_step).  After defer(), host arrays are mapped
    // without copying.  issue_in() copies the inputs, in map order, on a
    // copy stream; need(dev) makes the compute stream wait for that array's
    // copy (and so for every one mapped before it); put(dev) copies an
    // output back on a second copy stream once the compute stream has
    // written it for the last time; finish() puts the outputs not yet put,
    // joins both copy streams and synchronises.  Issued inside a stream
    // capture the copies become nodes of the graph: in_graph() then leaves
    // finish() only the synchronisation, and copy_out_all() copies every
    // output again on the compute stream (the host finished the step).
    void defer() { defer_ = true; }
    bool deferred() const { return defer_; }
    int issue_in();
    int need(const void *dev);
    int put(const void *dev);
    // put() of the output mapped to `dst` from the device array `src`,
    // which holds its final values already (the step copies src to dst
    // later without changing src)
    int put_as(const void *src, const void *dst);
    int put_rest();  // put() of every output not yet put
    int join();
    void clear_marks();
    void in_graph() { in_graph_ = true; }
    int copy_out_all();

  private:
    int map(const double *user, long n, bool out, double **dev, bool copy_in = true, long ncopy = -1);
    int event(int i, cudaEvent_t *e);
    Ctx *c_;
    const char *who_;
    cudaError_t pre_;
    struct Ent {
        const double *user;
        double *dev;
        long n;       // elements copied back (out)
        bool out;
        bool host;
        long nin = 0;     // elements copied in (deferred)
        int ev = -1;      // event of its deferred in-copy
        bool put = false; // deferred out-copy issued
    };
    std::vector<Ent> ent_;
    int slot_ = 0;
    bool any_host_ = false;
    bool pageable_ = false;
    bool defer_ = false, in_graph_ = false, forked_out_ = false, finished_ = false;
    int nev_ = 0;
};

} // namespace les
