// lester_phys_host.cu -- C ABI entry points of the momentum predictor and
// the scalar transport (include/lester_gpu.h).
#include <cstring>
#include <cuda.h>
#include <vector>
#include "kernels.h"
#include "lester_ctx.h"

namespace les {

// per-block tables of the predictor / scalar kernels, built on first use
static int ensure_phys_tables(Ctx &c)
{
    if (c.d_offki) return 0;
    int nb = c.g.numbl;
    std::vector<long> ki(nb), jk(nb);
    std::vector<int> link(6 * nb);
    long oki = 0, ojk = 0;
    int gm = 0;
    for (int b = 1; b <= nb; b++) {
        int *n = c.lv[1].n[b];
        ki[b - 1] = oki;
        jk[b - 1] = ojk;
        oki += (long)n[2] * n[0];
        ojk += (long)n[1] * n[2];
        for (int d = 0; d < 3; d++) gm = std::max(gm, n[d]);
        for (int s = 0; s < 6; s++) link[6 * (b - 1) + s] = c.g.bl2bl[b - 1][s] - 1;
    }
    LES_CUDA(cudaMalloc(&c.d_offki, sizeof(long) * nb));
    LES_CUDA(cudaMalloc(&c.d_offjk, sizeof(long) * nb));
    LES_CUDA(cudaMalloc(&c.d_link, sizeof(int) * 6 * nb));
    LES_CUDA(cudaMemcpy(c.d_offki, ki.data(), sizeof(long) * nb, cudaMemcpyHostToDevice));
    LES_CUDA(cudaMemcpy(c.d_offjk, jk.data(), sizeof(long) * nb, cudaMemcpyHostToDevice));
    LES_CUDA(cudaMemcpy(c.d_link, link.data(), sizeof(int) * 6 * nb, cudaMemcpyHostToDevice));
    c.gm = gm;
    c.gstride = (long)gm * gm;
    LES_CUDA(cudaMalloc(&c.d_grad, sizeof(double) * 6 * c.gstride * nb));
    LES_CUDA(cudaMemset(c.d_grad, 0, sizeof(double) * 6 * c.gstride * nb));
    long mf = 0;
    for (int b = 1; b <= nb; b++) {
        int *n = c.lv[1].n[b];
        long a = (long)(n[1] - 2) * (n[2] - 2), bq = (long)(n[0] - 2) * (n[2] - 2), cq = (long)(n[0] - 2) * (n[1] - 2);
        mf = std::max(mf, std::max(a, std::max(bq, cq)));
    }
    c.maxfacecell = mf;
    long l1 = 0;
    for (int b = 1; b <= nb; b++) l1 += (long)c.lv[1].n[b][0] * c.lv[1].n[b][1];
    c.tot2_l1 = l1;
    // planes i + j + k = s of the in-place scalar sweep
    std::vector<int2> sl;
    for (int b = 1; b <= nb; b++)
        for (int k = 2; k <= c.lv[1].n[b][2] - 1; k++) sl.push_back(make_int2(b - 1, k));
    int smin = 6, smax = 0;
    for (int b = 1; b <= nb; b++) smax = std::max(smax, c.lv[1].n[b][0] + c.lv[1].n[b][1] + c.lv[1].n[b][2] - 3);
    int ns = (int)sl.size();
    std::vector<int> cum((size_t)(smax - smin + 1) * (ns + 1));
    for (int sp = smin; sp <= smax; sp++) {
        int *row = &cum[(size_t)(sp - smin) * (ns + 1)];
        row[0] = 0;
        for (int q = 0; q < ns; q++) {
            const int *n = c.lv[1].n[sl[q].x + 1];
            int k = sl[q].y, ni = n[0] - 1, nj = n[1] - 1;
            int jlo = std::max(2, sp - k - ni), jhi = std::min(nj, sp - k - 2);
            row[q + 1] = row[q] + std::max(0, jhi - jlo + 1);
        }
    }
    c.nslice = ns;
    LES_CUDA(cudaMalloc(&c.d_wslice, sizeof(int2) * ns));
    LES_CUDA(cudaMemcpy(c.d_wslice, sl.data(), sizeof(int2) * ns, cudaMemcpyHostToDevice));
    LES_CUDA(cudaMalloc(&c.d_wcum, sizeof(int) * cum.size()));
    LES_CUDA(cudaMemcpy(c.d_wcum, cum.data(), sizeof(int) * cum.size(), cudaMemcpyHostToDevice));
    LES_CUDA(cudaMalloc(&c.d_wave, sizeof(WaveSync)));
    return 0;
}

// physics build of the current controls: 0 exact, 1 fast, 2 FP32
static int sweep_variant(const Ctx &c) { return c.c.exact ? 0 : phys32_on(c) ? 2 : 1; }

// Skew geometry of the tiled scalar sweep (k_sweep.cu), built on first use
static int ensure_sweep_geom(Ctx &c)
{
    Ctx::SweepState &W = c.sw;
    if (W.d_sb) return 0;
    const int nb = c.g.numbl;
    std::vector<SkewBlk> sb(nb);
    long s3 = 0, s2 = 0;
    for (int b = 1; b <= nb; b++) {
        SkewBlk &q = sb[b - 1];
        memset(&q, 0, sizeof q);
        const int *n = c.lv[1].n[b];
        for (int d = 0; d < 3; d++) {
            q.n[d] = n[d];
            W.maxn[d] = std::max(W.maxn[d], n[d]);
        }
        for (int s6 = 0; s6 < 6; s6++) q.bc[s6] = c.g.bl_bc[b - 1][s6];
        q.vp = (n[1] + 3) & ~3;
        q.off3 = c.lv[1].off3[b];
        q.off2 = c.lv[1].off2[b];
        q.off1k = c.lv[1].off1k[b];
        q.layer = (long)(n[0] + n[1] - 1) * q.vp;
        q.sk3 = s3;
        s3 += q.layer * n[2];
        q.sk2 = s2;
        s2 += q.layer;
    }
    W.tot3 = s3;
    W.tot2 = s2;
    LES_CUDA(cudaMalloc(&W.d_sb, sizeof(SkewBlk) * nb));
    LES_CUDA(cudaMemcpy(W.d_sb, sb.data(), sizeof(SkewBlk) * nb, cudaMemcpyHostToDevice));
    LES_CUDA(cudaMalloc(&W.d_sync, sizeof(int) * 2));  // ticket, error
    return 0;
}

// Tiles of build `var` (0 exact, 1 fast, 2 FP32), built on first use.  A
// block's interior rows are split into as few tiles as the build's ring
// allows (its shared memory grows with the rows of a tile; at most
// kSweepThreads rows); one tile per (block, interior layer k, row range),
// in ticket order (k, row range, block): every tile comes after the two
// whose new values it reads, (k-1, same rows) and (k, rows below).
static int ensure_sweep_tiles(Ctx &c, int var)
{
    Ctx::SweepState &W = c.sw;
    int r;
    if ((r = ensure_sweep_geom(c))) return r;
    if (W.d_tiles[var] || W.maxctas[var] < 0) return 0;
    const int nb = c.g.numbl;
    const int E = var == 2 ? 4 : 2;  // elements per 16-byte chunk
    // rows per tile: as many as kSweepThreads, with the ring for them (row
    // width rows + 4 halo rows + chunk rounding) within the 227 KB a CTA
    // may have
    auto smem_of = [&](int sw) {
        return var == 0 ? les_exact::sweep_tiles_smem(sw) : var == 1 ? les_fast::sweep_tiles_smem(sw)
                                                                     : les_f32::sweep_tiles_smem(sw);
    };
    int rows_max = kSweepThreads;
    while (rows_max >= 8 && smem_of(rows_max + 4 + 2 * E) > 227 * 1024 - 1024) rows_max--;
    if (rows_max < 8) {
        W.maxctas[var] = -1;
        return 0;
    }
    int maxk = 0, maxnj = 0;
    std::vector<int> nJ(nb);
    for (int b = 1; b <= nb; b++) {
        const int *n = c.lv[1].n[b];
        nJ[b - 1] = (n[1] - 2 + rows_max - 1) / rows_max;
        maxk = std::max(maxk, n[2]);
        maxnj = std::max(maxnj, nJ[b - 1]);
    }
    auto key = [&](int b, int k, int J) { return ((long)k * maxnj + J) * nb + b; };
    std::vector<int> idx((size_t)(maxk + 1) * maxnj * nb, -1);
    std::vector<SweepTile> tiles;
    int rows_big = 0;
    for (int k = 2; k < maxk; k++)
        for (int J = 0; J < maxnj; J++)
            for (int b = 0; b < nb; b++) {
                const int *n = c.lv[1].n[b + 1];
                if (k > n[2] - 1 || J >= nJ[b]) continue;
                const int rows = n[1] - 2, NJ = nJ[b];
                SweepTile T;
                T.blk = b;
                T.k = k;
                T.j0 = 2 + (int)((long)rows * J / NJ);
                T.j1 = 2 + (int)((long)rows * (J + 1) / NJ);
                T.up_k = k - 1 >= 2 ? idx[key(b, k - 1, J)] : -1;
                T.up_j = J > 0 ? idx[key(b, k, J - 1)] : -1;
                idx[key(b, k, J)] = (int)tiles.size();
                tiles.push_back(T);
                rows_big = std::max(rows_big, T.j1 - T.j0);
            }
    W.ntile[var] = (int)tiles.size();
    // ring row width: rows j0-2 .. j1+1 from a chunk boundary
    int w = 0;
    for (const SweepTile &T : tiles) {
        const int n1 = c.lv[1].n[T.blk + 1][1];
        const int sbase = (std::max(0, T.j0 - 3) / E) * E;
        const int hi = (std::min(n1, T.j1 + 1) + E - 1) / E * E;
        w = std::max(w, hi - sbase);
    }
    W.sw[var] = w;
    W.nthr[var] = 32 * ((rows_big + 31) / 32) + 32;  // row warps + the producer warp
    if (W.ntile[var] == 0) {
        W.maxctas[var] = -1;
        return 0;
    }
    LES_CUDA(cudaMalloc(&W.d_tiles[var], sizeof(SweepTile) * W.ntile[var]));
    LES_CUDA(cudaMemcpy(W.d_tiles[var], tiles.data(), sizeof(SweepTile) * W.ntile[var], cudaMemcpyHostToDevice));
    // occupancy with this ring (first use: never inside a capture, the
    // first step of a run is launched)
    const int n = var == 0 ? les_exact::sweep_tiles_max_ctas(w, W.nthr[var])
                  : var == 1 ? les_fast::sweep_tiles_max_ctas(w, W.nthr[var])
                             : les_f32::sweep_tiles_max_ctas(w, W.nthr[var]);
    W.maxctas[var] = n > 0 ? n : -1;
    return 0;
}

// TMA tensor maps of build `var` over the skewed copies of storage q (0
// FP64, 1 FP32), built once the copies exist: per block, the 3-D fields as
// (rows, planes of all layers, fields) in boxes of 8, 4 and 1 fields of
// one plane, and the ntab 2-D tables as (rows, planes, tables).  The map
// encoder is the driver's, reached through the runtime.
typedef CUresult (*PfnEncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int ensure_tensor_maps(Ctx &c, int var, int q, int ntab)
{
    Ctx::SweepState &W = c.sw;
    if (W.d_tmaps[var]) return 0;
    static PfnEncodeTiled encode = nullptr;
    if (!encode) {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult qr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &qr) != cudaSuccess ||
            qr != cudaDriverEntryPointSuccess || !f) {
            cudaGetLastError();
            return set_err(LES_ERR_CUDA, "set_sc1: cuTensorMapEncodeTiled unavailable");
        }
        encode = (PfnEncodeTiled)f;
    }
    const int nb = c.g.numbl;
    const size_t es = q == 1 ? sizeof(float) : sizeof(double);
    const CUtensorMapDataType dt = q == 1 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    char *base = (char *)W.d_sk[q];
    const cuuint32_t sw = (cuuint32_t)W.sw[var];
    std::vector<CUtensorMap> maps(4 * nb);
    for (int b = 1; b <= nb; b++) {
        const int *n = c.lv[1].n[b];
        const cuuint64_t vp = (cuuint64_t)((n[1] + 3) & ~3), np = (cuuint64_t)(n[0] + n[1] - 1);
        // the block's offsets in the skewed arrays (as ensure_sweep_geom lays them out)
        long sk3 = 0, sk2 = 0;
        for (int q2 = 1; q2 < b; q2++) {
            const int *m = c.lv[1].n[q2];
            const long lay = (long)(m[0] + m[1] - 1) * ((m[1] + 3) & ~3);
            sk3 += lay * m[2];
            sk2 += lay;
        }
        const cuuint64_t dim3[3] = {vp, np * (cuuint64_t)n[2], 9};
        const cuuint64_t str3[2] = {vp * es, (cuuint64_t)W.tot3 * es};
        const cuuint32_t estr[3] = {1, 1, 1};
        const cuuint32_t nf[3] = {8, 4, 1};
        for (int m = 0; m < 3; m++) {
            const cuuint32_t box[3] = {sw, 1, nf[m]};
            CUresult e = encode(&maps[4 * (b - 1) + m], dt, 3, base + es * sk3, dim3, str3, box, estr,
                                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (e != CUDA_SUCCESS) return set_err(LES_ERR_CUDA, "set_sc1: tensor map (block %d): error %d", b, (int)e);
        }
        const cuuint64_t dim2[3] = {vp, np, (cuuint64_t)ntab};
        const cuuint64_t str2[2] = {vp * es, (cuuint64_t)W.tot2 * es};
        const cuuint32_t box2[3] = {sw, 1, (cuuint32_t)ntab};
        CUresult e = encode(&maps[4 * (b - 1) + 3], dt, 3, base + es * (9 * W.tot3 + sk2), dim2, str2, box2, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (e != CUDA_SUCCESS) return set_err(LES_ERR_CUDA, "set_sc1: tensor map of the tables (block %d): error %d", b, (int)e);
    }
    LES_CUDA(cudaMalloc(&W.d_tmaps[var], sizeof(CUtensorMap) * maps.size()));
    LES_CUDA(cudaMemcpy(W.d_tmaps[var], maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice));
    return 0;
}

// Which scalar sweep runs (ctrl.sc1_sweep): 1 the hyperplane sweep, 2 the
// tile pipeline, 3 one launch per plane; 0 the tile pipeline for the FP32
// physics build where its ring fits, else the hyperplane sweep (with FP64
// arithmetic the hyperplane sweep, which spreads each plane over every SM,
// is the faster: GB300's FP64 rate bounds both, 8.0 against 10.0 ms on the
// 256x192x128 mixing layer).  Negative: an error.
static int sweep_choice(Ctx &c)
{
    const int m = c.c.sc1_sweep;
    if (m == 1 || m == 3) return m;
    if (m == 0 && !phys32_on(c)) return 1;
    const int var = sweep_variant(c);
    int r;
    if ((r = ensure_sweep_tiles(c, var))) return r;
    const bool fits = c.sw.maxctas[var] > 0;
    if (m == 2 && !fits) return set_err(LES_ERR_SIZE, "set_sc1: the tile pipeline's shared-memory ring does not fit");
    return fits ? 2 : 1;
}

// The tile pipeline on skewed copies of storage type S (q = 0 FP64, 1 FP32)
template <typename S>
static int run_sweep_tiles(Ctx &c, const Sc1Args &A, const double *const *rtab, const double *rdkp, int q,
                           void (*skew)(const SkewBlk *, int, int, int, int, int, const SkewPtrs<S> &, int,
                                        cudaStream_t),
                           void (*unskew)(const SkewBlk *, int, int, int, int, const S *, const S *, double *,
                                          double *, cudaStream_t),
                           void (*init_new)(const SkewBlk *, int, const S *, S *, cudaStream_t),
                           cudaError_t (*launch)(const SweepArgs<S> &, double, long, int, int, cudaStream_t))
{
    Ctx::SweepState &W = c.sw;
    const int nb = c.g.numbl;
    const bool fast = !c.c.exact;
    const int var = sweep_variant(c);
    int r;
    if (!W.d_sk[q]) {
        const size_t bytes = sizeof(S) * (9 * W.tot3 + 10 * W.tot2);
        if (cudaMalloc(&W.d_sk[q], bytes) != cudaSuccess) {
            cudaGetLastError();
            W.d_sk[q] = nullptr;
            return set_err(LES_ERR_NOMEM, "set_sc1: skewed copies (%zu bytes)", bytes);
        }
    }
    S *base = (S *)W.d_sk[q];
    SkewPtrs<S> P3, P2;
    memset(&P3, 0, sizeof P3);
    memset(&P2, 0, sizeof P2);
    const double *f3[8] = {A.sc1, A.hsc1, A.u, A.v, A.w, A.rho, A.gamsc1, A.gamlam};
    for (int f = 0; f < 8; f++) {
        P3.src[f] = f3[f];
        P3.dst[f] = base + f * W.tot3;
    }
    const double *f2[10] = {A.m[MW_DIU], A.m[MW_DJV], A.m[MW_RDJU], A.m[MW_RDIV], A.m[MW_RP],
                            A.m[MW_DIDJP], A.m[MW_RDIDJP], rtab[0], rtab[1], rtab[2]};
    const int n2 = fast ? 10 : 7;
    for (int f = 0; f < n2; f++) {
        P2.src[f] = f2[f];
        P2.dst[f] = base + 9 * W.tot3 + f * W.tot2;
    }
    skew(W.d_sb, nb, W.maxn[0], W.maxn[1], W.maxn[2], 8, P3, 0, c.stream);
    skew(W.d_sb, nb, W.maxn[0], W.maxn[1], W.maxn[2], n2, P2, 1, c.stream);
    SweepArgs<S> a;
    memset(&a, 0, sizeof a);
    a.sb = W.d_sb;
    a.tiles = W.d_tiles[var];
    a.ntile = W.ntile[var];
    a.sw = W.sw[var];
    for (int f = 0; f < 8; f++) a.f3[f] = P3.dst[f];
    for (int f = 0; f < n2; f++) a.f2[f] = P2.dst[f];
    a.dkp = A.dkp;
    a.dkw = A.dkw;
    a.rdkp = rdkp;
    a.grad = A.grad;
    a.gstride = A.gstride;
    a.gm = A.gm;
    a.link = A.link;
    a.scnew = base + 8 * W.tot3;
    a.ticket = W.d_sync;
    a.err = W.d_sync + 1;
    if ((r = ensure_tensor_maps(c, var, q, fast ? 10 : 7))) return r;
    a.tmaps = W.d_tmaps[var];
    init_new(W.d_sb, nb, P3.dst[0], a.scnew, c.stream);
    LES_CUDA(cudaMemsetAsync(W.d_sync, 0, sizeof(int) * 2, c.stream));
    const int nctas = std::min(W.ntile[var], W.maxctas[var]);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (c.prof && !c.capturing) {
        prof_pair(c, LES_PROF_SWEEP, &e0, &e1);
        cudaEventRecord(e0, c.stream);
    }
    LES_CUDA(launch(a, c.c.dtime, wait_polls(c), nctas, W.nthr[var], c.stream));
    if (e1) cudaEventRecord(e1, c.stream);
    unskew(W.d_sb, nb, W.maxn[0], W.maxn[1], W.maxn[2], a.scnew, P3.dst[1], A.sc1, A.hsc1, c.stream);
    if (c.capturing) {
        // a replayed step reads the wait's flag with its other status
        launch_copy_flag(a.err, c.d_loop + 6, c.stream);
    } else {
        int err = 0;
        LES_CUDA(cudaMemcpyAsync(&err, a.err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        LES_CUDA(cudaStreamSynchronize(c.stream));
        if (err) return set_err(LES_ERR_TIMEOUT, "set_sc1: a tile of the scalar sweep timed out waiting for a new value");
    }
    return 0;
}

static int sweep_tiles(Ctx &c, const Sc1Args &A, const double *const *rtab, const double *rdkp)
{
    if (phys32_on(c))
        return run_sweep_tiles<float>(c, A, rtab, rdkp, 1, les_f32::launch_sweep_skew, les_f32::launch_sweep_unskew,
                                      les_f32::launch_sweep_init_new, les_f32::launch_sweep_tiles);
    if (c.c.exact)
        return run_sweep_tiles<double>(c, A, rtab, rdkp, 0, les_exact::launch_sweep_skew,
                                       les_exact::launch_sweep_unskew, les_exact::launch_sweep_init_new,
                                       les_exact::launch_sweep_tiles);
    return run_sweep_tiles<double>(c, A, rtab, rdkp, 0, les_fast::launch_sweep_skew, les_fast::launch_sweep_unskew,
                                   les_fast::launch_sweep_init_new, les_fast::launch_sweep_tiles);
}

static int wave_range(Ctx &c, int &smin, int &smax)
{
    smin = 6;
    smax = 0;
    for (int b = 1; b <= c.g.numbl; b++) smax = std::max(smax, c.lv[1].n[b][0] + c.lv[1].n[b][1] + c.lv[1].n[b][2] - 3);
    return 0;
}

} // namespace les

namespace les {

void tab_reset(Ctx &c) { c.tab_next = 0; }

void phys32_reset(Ctx &c)
{
    // in a scope the pool keeps its copies while one entry point's worth of
    // room is left (the predictor's: 28 + 8 2-D tables, 4 1-D, 7 fields);
    // otherwise it starts again and forgets them
    const long reserve = 40 * c.tot2 + 8 * c.tot1k + 7 * (c.tot_sg3 + 4) + 64;
    if (!c.f32_scope || c.cap32 - c.next32 < reserve) {
        c.next32 = 0;
        c.f32_cache.clear();
    }
}

int phys32_tables(Ctx &c, int n, const double **const *pp, long len)
{
    if (!c.d_pool32) {
        // room for the three predictor calls of one step (f32_scope): the
        // metric tables they read, their per-call reciprocal tables, the
        // seven fields once
        const long cap = 96 * c.tot2 + 48 * c.tot1k + 7 * (c.tot_sg3 + 4) + 256;
        if (cudaMalloc(&c.d_pool32, sizeof(float) * cap) != cudaSuccess) {
            cudaGetLastError();
            return set_err(LES_ERR_NOMEM, "FP32 physics tables: %ld floats", cap);
        }
        c.cap32 = cap;
    }
    const double *src[64];
    float *dst[64];
    int m = 0;
    if (n > 64) return set_err(LES_ERR_ARG, "phys32_tables: %d tables", n);
    for (int t = 0; t < n; t++) {
        const double *q = *pp[t];
        if (!q || ((unsigned long long)q & 1ull)) continue;  // absent, or already a copy
        // tables made per call (the reciprocal and delta tables of the
        // fast builds) reuse their pool from call to call with other
        // contents: never taken from, or put in, the cache
        const bool pooled = c.d_tabpool && q >= c.d_tabpool && q < c.d_tabpool + c.tabcap;
        if (c.f32_scope && !pooled) {
            const float *hit = nullptr;
            for (const Ctx::F32Copy &e : c.f32_cache)
                if (e.src == q && e.len == len) hit = e.dst;
            if (hit) {
                *pp[t] = (const double *)((unsigned long long)hit | 1ull);
                continue;
            }
        }
        const long step = (len + 3) & ~3L;                   // 16-byte aligned copies
        if (c.next32 + step > c.cap32) return set_err(LES_ERR_SIZE, "FP32 physics tables exhausted");
        float *d = c.d_pool32 + c.next32;
        c.next32 += step;
        src[m] = q;
        dst[m] = d;
        m++;
        if (c.f32_scope && !pooled) c.f32_cache.push_back({q, len, d});
        *pp[t] = (const double *)((unsigned long long)d | 1ull);
    }
    if (m) launch_to_f32(src, dst, m, len, c.stream);
    return 0;
}

static int tab_take(Ctx &c, long len, double **p)
{
    if (!c.d_tabpool) {
        long cap = 24 * c.tot2 + 12 * c.tot1k;
        if (cudaMalloc(&c.d_tabpool, sizeof(double) * cap) != cudaSuccess) {
            cudaGetLastError();
            return set_err(LES_ERR_NOMEM, "fast physics tables: %ld doubles", cap);
        }
        c.tabcap = cap;
    }
    if (c.tab_next + len > c.tabcap) return set_err(LES_ERR_SIZE, "fast physics tables exhausted");
    *p = c.d_tabpool + c.tab_next;
    c.tab_next += len;
    return 0;
}

int recip_tabs(Ctx &c, int n, const double *const *src, long len, const double **out)
{
    double *dst[32];
    if (n > 32) return set_err(LES_ERR_ARG, "recip_tabs: %d tables", n);
    int r;
    for (int t = 0; t < n; t++) {
        if ((r = tab_take(c, len, &dst[t]))) return r;
        out[t] = dst[t];
    }
    launch_recip(src, dst, n, len, c.stream);
    return 0;
}

int delta_tabs(Ctx &c, const double *dip, const double *djp, const double *rp, const double *dkp,
               const double **d2, const double **d1)
{
    double *a, *b;
    int r;
    if ((r = tab_take(c, c.tot2, &a)) || (r = tab_take(c, c.tot1k, &b))) return r;
    launch_delta_tables(dip, djp, rp, c.tot2, dkp, c.tot1k, a, b, c.stream);
    *d2 = a;
    *d1 = b;
    return 0;
}

int fast_sgs_tabs(Ctx &c, const double *dip, const double *djp, const double *rp, const double *dkp,
                  const double *dkw, SgsFast &F)
{
    tab_reset(c);
    const double *src2[3] = {dip, djp, rp}, *o2[3], *o1[2];
    const double *src1[2] = {dkp, dkw};
    int r;
    if ((r = recip_tabs(c, 3, src2, c.tot2, o2)) || (r = recip_tabs(c, 2, src1, c.tot1k, o1)) ||
        (r = delta_tabs(c, dip, djp, rp, dkp, &F.delta2d, &F.delta1d)))
        return r;
    F.r_dip = o2[0];
    F.r_djp = o2[1];
    F.r_rp = o2[2];
    F.r_dkp = o1[0];
    F.r_dkw = o1[1];
    return 0;
}

} // namespace les

using namespace les;

extern "C" {

int lester_gpu_set_body_force(const double *fu, const double *fv, const double *fw)
{
    LES_NEED_CTX();
    const double *f[3] = {fu, fv, fw};
    for (int q = 0; q < 3; q++) {
        if (!f[q]) continue;
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, f[q]) != cudaSuccess ||
            (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
            cudaGetLastError();
            return set_err(LES_ERR_ARG, "body force %d must be device memory", q);
        }
    }
    for (int q = 0; q < 3; q++) g_ctx->fb[q] = f[q];
    return 0;
}

int lester_gpu_set_iststep(int iststep)
{
    LES_NEED_CTX();
    if (iststep < 1) return set_err(LES_ERR_ARG, "iststep must be >= 1");
    g_ctx->iststep = iststep;
    return 0;
}

// code/set_uv_int.F:5-164
int lester_set_uv_int(const int *iva, const double *u, const double *v, const double *w, const double *p,
                      const double *rho, const double *rhonp1, const double *gam, double *u_int, double *hu,
                      const double *dip, const double *diu, const double *dix, const double *rdix,
                      const double *djp, const double *dju, const double *djv, const double *djx,
                      const double *rdjp, const double *rdju, const double *didjp, const double *didju,
                      const double *rdidju, const double *hijp, const double *hiju, const double *hjiu,
                      const double *hkiu, const double *hkju, const double *rp, const double *ru,
                      const double *dkp, const double *dkw, double *tw_sfi, double *tw_nfi, double *tw_lfi,
                      double *tw_rfi, double *work, int *offwork)
{
    (void)work;
    (void)offwork;
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    int r;
    if ((r = ensure_phys_tables(c))) return r;
    int iv = *iva;
    if (iv != 1 && iv != 2) return set_err(LES_ERR_ARG, "set_uv_int: iva %d", iv);
    Staging st(&c, __func__);
    UIntArgs A;
    memset(&A, 0, sizeof A);
    const double *mu[20] = {dip, diu, dix, rdix, djp, dju, djv, djx, rdjp, rdju,
                            didjp, didju, rdidju, hijp, hiju, hjiu, hkiu, hkju, rp, ru};
    const double **md[20] = {&A.dip, &A.diu, &A.dix, &A.rdix, &A.djp, &A.dju, &A.djv, &A.djx, &A.rdjp,
                             &A.rdju, &A.didjp, &A.didju, &A.rdidju, &A.hijp, &A.hiju, &A.hjiu, &A.hkiu,
                             &A.hkju, &A.rp, &A.ru};
    for (int q = 0; q < 20; q++)
        if ((r = st.in(mu[q], c.tot2, md[q]))) return r;
    if ((r = st.in(dkp, c.tot1k, &A.dkp)) || (r = st.in(dkw, c.tot1k, &A.dkw))) return r;
    const double *fu[7] = {u, v, w, p, rho, rhonp1, gam};
    const double **fd[7] = {&A.u, &A.v, &A.w, &A.p, &A.rho, &A.rhonp1, &A.gam};
    for (int q = 0; q < 7; q++)
        if ((r = st.in(fu[q], c.tot_sg3, fd[q]))) return r;
    if ((r = st.io(u_int, c.tot_sg3, &A.u_int)) || (r = st.io(hu, c.tot_sg3, &A.hu))) return r;
    long nsn = (iv == 1) ? c.totki : c.totjk;
    if ((r = st.io(tw_sfi, nsn, &A.tw_s)) || (r = st.io(tw_nfi, nsn, &A.tw_n)) ||
        (r = st.io(tw_lfi, c.tot2_l1, &A.tw_l)) || (r = st.io(tw_rfi, c.tot2_l1, &A.tw_r)))
        return r;
    A.off_ki = c.d_offki;
    A.off_jk = c.d_offjk;
    A.off2_lev1_base = 0;
    A.fb = c.fb[iv - 1];
    A.iststep = c.capturing ? c.d_step : nullptr;
    const lester_ctrl &k = c.c;
    LevelGeom &L = c.lv[1];
    if (!k.exact) {
        tab_reset(c);
        const double *src2[8] = {A.dip, A.diu, A.dix, A.djp, A.dju, A.djv, A.djx, A.rp};
        const double **dst2[8] = {&A.r_dip, &A.r_diu, &A.r_dix, &A.r_djp, &A.r_dju, &A.r_djv, &A.r_djx, &A.r_rp};
        const double *src1[2] = {A.dkp, A.dkw};
        const double *o2[8], *o1[2];
        if ((r = recip_tabs(c, 8, src2, c.tot2, o2)) || (r = recip_tabs(c, 2, src1, c.tot1k, o1))) return r;
        for (int q = 0; q < 8; q++) *dst2[q] = o2[q];
        A.r_dkp = o1[0];
        A.r_dkw = o1[1];
    }
    if (phys32_on(c)) {
        phys32_reset(c);
        const double **const t2[28] = {&A.dip, &A.diu, &A.dix, &A.rdix, &A.djp, &A.dju, &A.djv, &A.djx, &A.rdjp,
                                       &A.rdju, &A.didjp, &A.didju, &A.rdidju, &A.hijp, &A.hiju, &A.hjiu, &A.hkiu,
                                       &A.hkju, &A.rp, &A.ru, &A.r_dip, &A.r_diu, &A.r_dix, &A.r_djp, &A.r_dju,
                                       &A.r_djv, &A.r_djx, &A.r_rp};
        const double **const t1[4] = {&A.dkp, &A.dkw, &A.r_dkp, &A.r_dkw};
        const double **const t3[7] = {&A.u, &A.v, &A.w, &A.p, &A.rho, &A.rhonp1, &A.gam};
        if ((r = phys32_tables(c, 28, t2, c.tot2)) || (r = phys32_tables(c, 4, t1, c.tot1k)) ||
            (r = phys32_tables(c, 7, t3, c.tot_sg3)))
            return r;
    }
    LES_PHYS(c, launch_set_u_int)(L.d_blk, c.g.numbl, L.maxcell, iv, A, k.dtime, c.iststep, k.visc, k.ylaminar,
                                  k.kappa, k.cwfun, c.stream);
    launch_halo(L.d_face, L.nface, L.maxface, A.u_int, c.d_work, c.stream);
    return st.finish();
}

// code/set_w_int.F:5-141
int lester_set_w_int(const double *u, const double *v, const double *w, const double *p, const double *rho,
                     const double *rhonp1, const double *gam, double *w_int, double *hw, const double *dip,
                     const double *diu, const double *rdiv, const double *djp, const double *djv,
                     const double *rdju, const double *didjp, const double *rdidjp, const double *hkip,
                     const double *hkjp, const double *hkiu, const double *hkjv, const double *rp,
                     const double *ru, const double *dkp, const double *dkw, double *tw_sfk, double *tw_nfk,
                     double *tw_wfk, double *tw_efk, double *work, int *offwork)
{
    (void)work;
    (void)offwork;
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    int r;
    if ((r = ensure_phys_tables(c))) return r;
    Staging st(&c, __func__);
    WIntArgs A;
    memset(&A, 0, sizeof A);
    const double *mu[MW_N] = {dip, diu, rdiv, djp, djv, rdju, didjp, rdidjp, hkip, hkjp, hkiu, hkjv, rp, ru};
    for (int q = 0; q < MW_N; q++)
        if ((r = st.in(mu[q], c.tot2, &A.m[q]))) return r;
    if ((r = st.in(dkp, c.tot1k, &A.dkp)) || (r = st.in(dkw, c.tot1k, &A.dkw))) return r;
    const double *fu[7] = {u, v, w, p, rho, rhonp1, gam};
    const double **fd[7] = {&A.u, &A.v, &A.w, &A.p, &A.rho, &A.rhonp1, &A.gam};
    for (int q = 0; q < 7; q++)
        if ((r = st.in(fu[q], c.tot_sg3, fd[q]))) return r;
    if ((r = st.io(w_int, c.tot_sg3, &A.w_int)) || (r = st.io(hw, c.tot_sg3, &A.hw))) return r;
    if ((r = st.io(tw_sfk, c.totki, &A.tw_sfk)) || (r = st.io(tw_nfk, c.totki, &A.tw_nfk)) ||
        (r = st.io(tw_wfk, c.totjk, &A.tw_wfk)) || (r = st.io(tw_efk, c.totjk, &A.tw_efk)))
        return r;
    A.off_ki = c.d_offki;
    A.off_jk = c.d_offjk;
    A.fb = c.fb[2];
    A.iststep = c.capturing ? c.d_step : nullptr;
    const lester_ctrl &k = c.c;
    LevelGeom &L = c.lv[1];
    if (!k.exact) {
        tab_reset(c);
        const int qs[5] = {MW_DIU, MW_DJV, MW_RP, MW_DJP, MW_DIP};
        const double *src2[5], *o2[5], *o1[2];
        for (int t = 0; t < 5; t++) src2[t] = A.m[qs[t]];
        const double *src1[2] = {A.dkp, A.dkw};
        if ((r = recip_tabs(c, 5, src2, c.tot2, o2)) || (r = recip_tabs(c, 2, src1, c.tot1k, o1))) return r;
        for (int t = 0; t < 5; t++) A.r[qs[t]] = o2[t];
        A.rdkp = o1[0];
        A.rdkw = o1[1];
    }
    if (phys32_on(c)) {
        phys32_reset(c);
        const double **t2[2 * MW_N];
        for (int q = 0; q < MW_N; q++) {
            t2[q] = &A.m[q];
            t2[MW_N + q] = &A.r[q];
        }
        const double **const t1[4] = {&A.dkp, &A.dkw, &A.rdkp, &A.rdkw};
        const double **const t3[7] = {&A.u, &A.v, &A.w, &A.p, &A.rho, &A.rhonp1, &A.gam};
        if ((r = phys32_tables(c, 2 * MW_N, t2, c.tot2)) || (r = phys32_tables(c, 4, t1, c.tot1k)) ||
            (r = phys32_tables(c, 7, t3, c.tot_sg3)))
            return r;
    }
    LES_PHYS(c, launch_set_w_int)(L.d_blk, c.g.numbl, L.maxcell, A, k.dtime, c.iststep, k.visc, k.ylaminar,
                                  k.kappa, k.cwfun, c.stream);
    launch_halo(L.d_face, L.nface, L.maxface, A.w_int, c.d_work, c.stream);
    return st.finish();
}

// code/set_virt_bc.F:8 set_virt_bc(iva, ilev, f, fm, rho, gam, vd_damping,
// init_vdd, value, tw_sfi ... tw_nfk, dip, diu, div, dix, djp, dju, djv,
// djx, ru, rv, dkp, dkw) at ilev = 1 for the velocities.  init_vdd is kept
// by the library (set for every side by the u call); the argument is
// accepted and ignored.
int lester_set_virt_bc(const int *iva, const int *ilev, double *f, const double *fm, const double *rho,
                       const double *gam, double *vd_damping, int *init_vdd, const double *value,
                       double *tw_sfi, double *tw_nfi, double *tw_lfi, double *tw_rfi, double *tw_wfj,
                       double *tw_efj, double *tw_lfj, double *tw_rfj, double *tw_wfk, double *tw_efk,
                       double *tw_sfk, double *tw_nfk, const double *dip, const double *diu,
                       const double *div, const double *dix, const double *djp, const double *dju,
                       const double *djv, const double *djx, const double *ru, const double *rv,
                       const double *dkp, const double *dkw)
{
    (void)fm;
    (void)gam;
    (void)init_vdd;
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    int r;
    if ((r = ensure_phys_tables(c))) return r;
    int iv = *iva;
    if (iv < 1 || iv > 3 || *ilev != 1) return set_err(LES_ERR_ARG, "set_virt_bc: velocities at level 1 only");
    Staging st(&c, __func__);
    VbcArgs A;
    memset(&A, 0, sizeof A);
    if ((r = st.io(f, c.tot_sg3, &A.f)) || (r = st.in(rho, c.tot_sg3, &A.rho)) ||
        (r = st.io(vd_damping, c.tot_sg3, &A.vdd)))
        return r;
    const double *mu[10] = {dju, djx, ru, rv, div, dix, dip, diu, djp, djv};
    const double **md[10] = {&A.dju, &A.djx, &A.ru, &A.rv, &A.div_, &A.dix, &A.dip, &A.diu, &A.djp, &A.djv};
    for (int q = 0; q < 10; q++)
        if ((r = st.in(mu[q], c.tot2, md[q]))) return r;
    if ((r = st.in(dkp, c.tot1k, &A.dkp)) || (r = st.in(dkw, c.tot1k, &A.dkw))) return r;
    // the four wall arrays of this component and their layouts
    double *tws[4];
    long twn[4];
    if (iv == 1) {
        double *t[4] = {tw_sfi, tw_nfi, tw_lfi, tw_rfi};
        long n[4] = {c.totki, c.totki, c.tot2_l1, c.tot2_l1};
        for (int q = 0; q < 4; q++) { tws[q] = t[q]; twn[q] = n[q]; }
    } else if (iv == 2) {
        double *t[4] = {tw_wfj, tw_efj, tw_lfj, tw_rfj};
        long n[4] = {c.totjk, c.totjk, c.tot2_l1, c.tot2_l1};
        for (int q = 0; q < 4; q++) { tws[q] = t[q]; twn[q] = n[q]; }
    } else {
        double *t[4] = {tw_wfk, tw_efk, tw_sfk, tw_nfk};
        long n[4] = {c.totjk, c.totjk, c.totki, c.totki};
        for (int q = 0; q < 4; q++) { tws[q] = t[q]; twn[q] = n[q]; }
    }
    double *twd[4] = {nullptr, nullptr, nullptr, nullptr};
    A.off_ki = c.d_offki;
    A.off_jk = c.d_offjk;
    int nb = c.g.numbl;
    if (iv == 1)
        for (int b = 0; b < nb; b++)
            for (int s = 0; s < 6; s++) c.init_vdd[b][s] = 1;
    les_exact::launch_fill(A.vdd, 1.0, c.tot_sg3, c.stream);
    // sides this component treats (set_virt_bc.F:77-135): not its own axis
    const int sides[3][4] = {{3, 4, 5, 6}, {1, 2, 5, 6}, {1, 2, 3, 4}};
    for (int q = 0; q < 4; q++) {
        int s = sides[iv - 1][q];
        unsigned long long wall = 0, init = 0;
        long maxpts = 0;
        for (int b = 1; b <= nb; b++) {
            if (c.g.bl_bc[b - 1][s - 1] != LES_BCT_WALL) continue;
            wall |= 1ull << (b - 1);
            if (c.init_vdd[b - 1][s - 1]) init |= 1ull << (b - 1);
            c.init_vdd[b - 1][s - 1] = 0;
            int *n = c.lv[1].n[b];
            long pts;
            if (iv == 1 && (s == 3 || s == 4)) pts = (long)n[0] * n[2] * (n[1] / 2 + 1);
            else if (s <= 2) pts = (long)n[1] * n[2];
            else if (s <= 4) pts = (long)n[0] * n[2];
            else pts = (long)n[0] * n[1];
            maxpts = std::max(maxpts, pts);
        }
        if (!wall) continue;
        if (!twd[q] && (r = st.io(tws[q], twn[q], &twd[q]))) return r;
        A.tw = twd[q];
        launch_vbc_side(c.lv[1].d_blk, nb, iv, s, wall, init, A, maxpts, c.c.visc, c.c.kappa, c.c.aplus,
                        c.c.ylaminar, value ? *value : 0.0, c.stream);
    }
    return st.finish();
}

// code/set_gamsc1_bc.F
int lester_set_gamsc1_bc(const double *sc1, double *gamsc1, double *gamlam, const double *diu,
                         const double *djv, const double *dkp, const double *rp)
{
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    int r;
    if ((r = ensure_phys_tables(c))) return r;
    Staging st(&c, __func__);
    const double *ds, *ddiu, *ddjv, *ddkp, *drp;
    double *dg, *dl;
    if ((r = st.in(sc1, c.tot_sg3, &ds)) || (r = st.io(gamsc1, c.tot_sg3, &dg)) ||
        (r = st.io(gamlam, c.tot_sg3, &dl)) || (r = st.in(diu, c.tot2, &ddiu)) || (r = st.in(djv, c.tot2, &ddjv)) ||
        (r = st.in(dkp, c.tot1k, &ddkp)) || (r = st.in(rp, c.tot2, &drp)))
        return r;
    les_exact::launch_fill(dl, c.c.visc / 0.72, c.tot_sg3, c.stream);
    LevelGeom &L = c.lv[1];
    les_exact::launch_face_bc(L.d_blk, c.g.numbl, c.maxfacecell, 0, nullptr, dg, dl, ds, ddiu, ddjv, drp, ddkp, c.d_grad,
                   c.gstride, c.gm, c.stream);
    return st.finish();
}

// code/set_sc1.F:5-95
int lester_set_sc1(const double *u, const double *v, const double *w, const double *p, double *sc1,
                   const double *rho, const double *gamsc1, const double *gamlam, double *hsc1,
                   const double *dip, const double *diu, const double *rdiv, const double *djp,
                   const double *djv, const double *rdju, const double *didjp, const double *rdidjp,
                   const double *hkip, const double *hkjp, const double *hkiu, const double *hkjv,
                   const double *rp, const double *dkp, const double *dkw, double *work, int *offwork)
{
    (void)p;
    (void)work;
    (void)offwork;
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    int r;
    if ((r = ensure_phys_tables(c))) return r;
    Staging st(&c, __func__);
    Sc1Args A;
    memset(&A, 0, sizeof A);
    const double *mu[MW_N] = {dip, diu, rdiv, djp, djv, rdju, didjp, rdidjp, hkip, hkjp, hkiu, hkjv, rp, nullptr};
    for (int q = 0; q < MW_N; q++)
        if ((r = st.in(mu[q], c.tot2, &A.m[q]))) return r;
    if ((r = st.in(dkp, c.tot1k, &A.dkp)) || (r = st.in(dkw, c.tot1k, &A.dkw))) return r;
    const double *fu[6] = {u, v, w, rho, gamsc1, gamlam};
    const double **fd[6] = {&A.u, &A.v, &A.w, &A.rho, &A.gamsc1, &A.gamlam};
    for (int q = 0; q < 6; q++)
        if ((r = st.in(fu[q], c.tot_sg3, fd[q]))) return r;
    if ((r = st.io(sc1, c.tot_sg3, &A.sc1)) || (r = st.io(hsc1, c.tot_sg3, &A.hsc1))) return r;
    A.grad = c.d_grad;
    A.gstride = c.gstride;
    A.gm = c.gm;
    A.link = c.d_link;
    LevelGeom &L = c.lv[1];
    int smin, smax;
    wave_range(c, smin, smax);
    const double *rtab[3] = {nullptr, nullptr, nullptr}, *rdkp = nullptr;  // FP64 reciprocals (fast builds)
    if (!c.c.exact) {
        tab_reset(c);
        const double *src2[3] = {A.m[MW_DIU], A.m[MW_DJV], A.m[MW_RP]}, *o2[3], *o1[1];
        const double *src1[1] = {A.dkp};
        if ((r = recip_tabs(c, 3, src2, c.tot2, o2)) || (r = recip_tabs(c, 1, src1, c.tot1k, o1))) return r;
        A.r[MW_DIU] = o2[0];
        A.r[MW_DJV] = o2[1];
        A.r[MW_RP] = o2[2];
        A.rdkp = o1[0];
        for (int q = 0; q < 3; q++) rtab[q] = o2[q];
        rdkp = o1[0];
    }
    if ((r = sweep_choice(c)) < 0) return r;
    if (r == 2) {
        if ((r = sweep_tiles(c, A, rtab, rdkp))) return r;
        launch_halo(L.d_face, L.nface, L.maxface, A.sc1, c.d_work, c.stream);
        return st.finish();
    }
    if (phys32_on(c)) {
        phys32_reset(c);
        const double **t2[2 * MW_N];
        for (int q = 0; q < MW_N; q++) {
            t2[q] = &A.m[q];
            t2[MW_N + q] = &A.r[q];
        }
        const double **const t1[3] = {&A.dkp, &A.dkw, &A.rdkp};
        if ((r = phys32_tables(c, 2 * MW_N, t2, c.tot2)) || (r = phys32_tables(c, 3, t1, c.tot1k))) return r;
    }
    // the whole sweep as one cooperative launch with a grid barrier per
    // plane; per-plane launches where the device cannot co-schedule it
    int smem = (int)sizeof(int) * (c.nslice + 1);
    int maxctas = smem <= 48 * 1024 && c.c.sc1_sweep != 3 ? LES_PHYS(c, sc1_sweep_max_ctas)(smem) : 0;
    if (c.c.sc1_sweep == 1 && maxctas <= 0)
        return set_err(LES_ERR_SIZE, "set_sc1: the hyperplane sweep does not fit as one cooperative launch");
    if (maxctas > 0) {
        LES_CUDA(cudaMemsetAsync(c.d_wave, 0, sizeof(WaveSync), c.stream));
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (c.prof && !c.capturing) {
            prof_pair(c, LES_PROF_SWEEP, &e0, &e1);
            cudaEventRecord(e0, c.stream);
        }
        LES_CUDA(LES_PHYS(c, launch_sc1_sweep)(L.d_blk, c.d_wcum, c.d_wslice, c.nslice, maxctas, smin, smax, A,
                                               c.c.dtime, c.d_wave, wait_polls(c), c.stream));
        if (e1) cudaEventRecord(e1, c.stream);
        if (c.capturing) {
            // a replayed step reads the barrier's flag with its other status
            launch_copy_flag(&c.d_wave->err, c.d_loop + 6, c.stream);
        } else {
            int err = 0;
            LES_CUDA(cudaMemcpyAsync(&err, &c.d_wave->err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
            LES_CUDA(cudaStreamSynchronize(c.stream));
            if (err) return set_err(LES_ERR_TIMEOUT, "set_sc1: grid barrier of the scalar sweep timed out");
        }
    } else {
        LES_PHYS(c, launch_sc1_waves)(L.d_blk, c.g.numbl, L.maxjk, smin, smax, A, c.c.dtime, c.stream);
    }
    launch_halo(L.d_face, L.nface, L.maxface, A.sc1, c.d_work, c.stream);
    return st.finish();
}

// code/set_sc1_bc.F
int lester_set_sc1_bc(double *sc1)
{
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    int r;
    if ((r = ensure_phys_tables(c))) return r;
    Staging st(&c, __func__);
    double *d;
    if ((r = st.io(sc1, c.tot_sg3, &d))) return r;
    LevelGeom &L = c.lv[1];
    les_exact::launch_face_bc(L.d_blk, c.g.numbl, c.maxfacecell, 1, d, nullptr, nullptr, nullptr, nullptr, nullptr,
                   nullptr, nullptr, nullptr, 0, 0, c.stream);
    return st.finish();
}

// code/set_sc1var.F (sc1var only; the block routine does not write sc1dis)
int lester_set_sc1var(const double *u, const double *v, const double *w, const double *sc1, const double *rho,
                      double *sc1var, double *sc1dis, const double *dip, const double *djp, const double *dkp,
                      const double *dkw, const double *rp, double *work, int *offwork)
{
    (void)u;
    (void)v;
    (void)w;
    (void)rho;
    (void)sc1dis;
    (void)work;
    (void)offwork;
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    Staging st(&c, __func__);
    const double *ds, *ddip, *ddjp, *ddkp, *ddkw, *drp;
    double *dv;
    int r;
    if ((r = st.in(sc1, c.tot_sg3, &ds)) || (r = st.io(sc1var, c.tot_sg3, &dv)) || (r = st.in(dip, c.tot2, &ddip)) ||
        (r = st.in(djp, c.tot2, &ddjp)) || (r = st.in(dkp, c.tot1k, &ddkp)) || (r = st.in(dkw, c.tot1k, &ddkw)) ||
        (r = st.in(rp, c.tot2, &drp)))
        return r;
    LevelGeom &L = c.lv[1];
    SgsFast F;
    memset(&F, 0, sizeof F);
    if (!c.c.exact && (r = fast_sgs_tabs(c, ddip, ddjp, drp, ddkp, ddkw, F))) return r;
    if (phys32_on(c)) {
        phys32_reset(c);
        const double **const t2[6] = {&ddip, &ddjp, &drp, &F.r_dip, &F.r_djp, &F.r_rp};
        const double **const t2b[1] = {&F.delta2d};
        const double **const t1[5] = {&ddkp, &ddkw, &F.r_dkp, &F.r_dkw, &F.delta1d};
        if ((r = phys32_tables(c, 6, t2, c.tot2)) || (r = phys32_tables(c, 1, t2b, c.tot2)) ||
            (r = phys32_tables(c, 5, t1, c.tot1k)))
            return r;
    }
    LES_PHYS(c, launch_sc1var)(L.d_blk, c.g.numbl, L.maxcell, ds, dv, ddip, ddjp, drp, ddkp, ddkw, F, c.stream);
    launch_halo(L.d_face, L.nface, L.maxface, dv, c.d_work, c.stream);
    return st.finish();
}

} // extern "C"
