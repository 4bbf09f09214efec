// k_sweep.cu -- the in-place scalar update of set_sc1_block
// (code/set_sc1_block.F:104-502) as a pipeline of tiles.
//
// The update of sc1 at (i, j, k) reads sc1 at +-1 and +-2 along each axis
// only, new values on the minus side and old ones on the plus side (the
// reference's in-place loop).  Within one k layer the points of a plane
// t = i + j are independent given planes t-1, t-2 of the layer and plane t
// of the layers k-1, k-2 (new) and k+1, k+2 (old).  So:
//
//  * a tile is (block, layer k, rows j0..j1-1); one CTA walks its planes t
//    in order, one thread per row, a __syncthreads between planes;
//  * tile (k, J) needs the new values of plane t of layers k-1 and k-2 and
//    of planes t-1, t-2 of rows j0-1, j0-2 (tile (k, J-1)); every other
//    value it reads is an old one.  Old values come from a read-only skewed
//    copy of sc1; new values are written to a second skewed array whose
//    interior starts as a sentinel (-1, below the scalar's clamp at 0), so
//    a tile simply checks each new value it staged and re-reads it from L2
//    until it is no longer the sentinel (bounded).  No flags, no fences, no
//    anti-dependences: the tiles run as a wavefront one layer apart, in
//    ticket order (every tile waits only on tiles with smaller tickets);
//  * every field is first copied into a skewed layout (k_skew), in which
//    plane t of a layer is one contiguous vector over j, so a tile stages
//    the vectors of the planes it will need with coalesced 16-byte cp.async
//    copies into a shared-memory ring, D planes ahead; the new values go
//    to the new-value array and to the ring (read by later planes of the
//    tile) and are copied to the FP64 fields at the end (k_unskew).
//
// The arithmetic per point is that of sc1_cell in k_phys.cu, operand for
// operand, so the exact build (FP64, -fmad=false) equals the hyperplane
// sweep and the oracle bit for bit; the fast build uses the reciprocal
// metric tables (x * (1/d)) as k_phys.cu's fast build does; the FP32 build
// is the same template with R = S = float (FP64 fields in HBM, FP32 skewed
// copies).
#include "k_common.cuh"
#include "kernels.h"

#if defined(LES_SWEEP_EXACT)
#define SWEEP_NS les_exact
#else
#define SWEEP_NS les_fast
#endif

namespace les_sweep {
namespace {  // internal to each build of this unit

// vectors staged per plane: own layer (3-D fields 0..7), the layers k-1,
// k-2, k+1, k+2, and the 2-D metric tables (reciprocals last: fast only)
enum {
    V_SC, V_H, V_U, V_V, V_W, V_RHO, V_GS, V_GL,
    V_SCM1, V_RHOM1, V_GSM1, V_GLM1, V_SCM2,
    V_SCP1, V_RHOP1, V_GSP1, V_GLP1, V_WP1, V_SCP2,
    V_DIU, V_DJV, V_RDJU, V_RDIV, V_RP, V_DIDJP, V_RDIDJP,
    V_RDIU, V_RDJV, V_RRP,
    V_SCH,  // own layer, rows j0-2, j0-1 of the tile below (new values)
    V_N
};

// per vector: source (0..7 a 3-D field: sc1 hsc1 u v w rho gamsc1 gamlam;
// 8 + q the 2-D table q; 18 the new-value array), layer offset, and the
// plane window [t+lo, t+hi] a point of plane t reads.  SCM1 and SCM2 read
// the new-value array where their layer is an interior one.
struct VecDesc {
    int src, dk, lo, hi;
};
__host__ __device__ constexpr VecDesc vdesc(int v)
{
    constexpr VecDesc d[V_N] = {
        {0, 0, -2, 2}, {1, 0, 0, 0}, {2, 0, 0, 1}, {3, 0, 0, 1}, {4, 0, 0, 0}, {5, 0, -1, 1}, {6, 0, -1, 1},
        {7, 0, -1, 1},
        {0, -1, 0, 0}, {5, -1, 0, 0}, {6, -1, 0, 0}, {7, -1, 0, 0}, {0, -2, 0, 0},
        {0, 1, 0, 0}, {5, 1, 0, 0}, {6, 1, 0, 0}, {7, 1, 0, 0}, {4, 1, 0, 0}, {0, 2, 0, 0},
        {8, 0, -1, 2}, {9, 0, -1, 2}, {10, 0, 0, 1}, {11, 0, 0, 1}, {12, 0, 0, 0}, {13, 0, 0, 0},
        {14, 0, 0, 0},
        {15, 0, -1, 2}, {16, 0, -1, 2}, {17, 0, 0, 0},
        {18, 0, -2, -1}};
    return d[v];
}
// ring slots of vector v for prefetch distance D: planes t+lo .. t+hi+D,
// rounded up to a power of two so that a plane's slot is (p & (slots-1))
__host__ __device__ constexpr int pow2_ceil(int n) { return n <= 1 ? 1 : 2 * pow2_ceil((n + 1) / 2); }
__host__ __device__ constexpr int vslots(int v, int D) { return pow2_ceil(vdesc(v).hi - vdesc(v).lo + D + 1); }
// ring slots before vector v (compile time)
__host__ __device__ constexpr int vprefix(bool fast, int v, int D)
{
    int s = 0;
    for (int u = 0; u < v; u++)
        if (fast || u < V_RDIU || u > V_RRP) s += vslots(u, D);
    return s;
}
// vectors of a build: the exact build has no reciprocal tables
__host__ __device__ constexpr bool has_vec(bool fast, int v) { return fast || v < V_RDIU || v > V_RRP; }
__host__ __device__ constexpr int ring_slots(bool fast, int D)
{
    int s = 0;
    for (int v = 0; v < V_N; v++)
        if (has_vec(fast, v)) s += vslots(v, D);
    return s;
}

// the same table for lookups by a runtime vector index (the producer lane)
__constant__ VecDesc c_vdesc[V_N] = {
    {0, 0, -2, 2}, {1, 0, 0, 0}, {2, 0, 0, 1}, {3, 0, 0, 1}, {4, 0, 0, 0}, {5, 0, -1, 1}, {6, 0, -1, 1},
    {7, 0, -1, 1},
    {0, -1, 0, 0}, {5, -1, 0, 0}, {6, -1, 0, 0}, {7, -1, 0, 0}, {0, -2, 0, 0},
    {0, 1, 0, 0}, {5, 1, 0, 0}, {6, 1, 0, 0}, {7, 1, 0, 0}, {4, 1, 0, 0}, {0, 2, 0, 0},
    {8, 0, -1, 2}, {9, 0, -1, 2}, {10, 0, 0, 1}, {11, 0, 0, 1}, {12, 0, 0, 0}, {13, 0, 0, 0},
    {14, 0, 0, 0},
    {15, 0, -1, 2}, {16, 0, -1, 2}, {17, 0, 0, 0},
    {18, 0, -2, -1}};

template <bool FAST, int D> __device__ __forceinline__ int vprefix_rt(int v)
{
    int s = 0;
#pragma unroll
    for (int u = 0; u < V_N; u++)
        if (u < v && has_vec(FAST, u)) s += vslots(u, D);
    return s;
}

// the new-value array's initial value: the scalar is clamped to [0, 1]
constexpr float kSentinel = -1.0f;

__device__ __forceinline__ float ld_strong(const float *p)
{
    float v;
    asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ double ld_strong(const double *p)
{
    double v;
    asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_strong(float *p, float v)
{
    asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}
__device__ __forceinline__ void st_strong(double *p, double v)
{
    asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// A new value staged from the new-value array: while it is still the
// sentinel, re-read it from L2 (another CTA is computing it); bounded by
// `limit` polls, or until another CTA has set *err (then *err is set and
// the staged value returned: the call reports LES_ERR_TIMEOUT).
template <typename S>
__device__ S fresh(S v, const S *g, int *err, long limit)
{
    long it = 0;
    while (v == (S)kSentinel) {
        if (*(volatile int *)err) return v;
        if (++it > limit) {
            atomicExch(err, 1);
            return v;
        }
        __nanosleep(32);
        v = ld_strong(g);
    }
    return v;
}

// ------------------------------------------------------------------ skew
// Copy a 3-D field (or a 2-D table: n2 = 1) from the reference layout into
// the skewed layout through a 32 x 32 (plane, row) shared tile: coalesced
// reads along i, coalesced writes along j.  Element (i, j, k) goes to
// sk + (k-1) layer + (i+j-2) vp + (j-1); entries of a plane vector whose i
// falls outside 1..nip1 are not written.
template <typename S>
__global__ void __launch_bounds__(256) k_skew(const SkewBlk *__restrict__ sb, int nfield, SkewPtrs<S> P,
                                              int two_d, int ntp)
{
    __shared__ double tile[32][33];
    const SkewBlk b = sb[blockIdx.z / nfield];
    const int f = blockIdx.z % nfield;
    const int n0 = b.n[0], n1 = b.n[1];
    const int nlay = two_d ? 1 : b.n[2];
    const int k = blockIdx.y + 1;
    if (k > nlay) return;
    const int tt = blockIdx.x % ntp, jt = blockIdx.x / ntp;
    if (jt * 32 >= n1 || 32 * tt > n0 + n1 - 2) return;
    const int t0 = 2 + 32 * tt, jb = 1 + 32 * jt;
    const double *s = P.src[f] + (two_d ? b.off2 : b.off3 + (long)n0 * n1 * (k - 1));
    S *d = P.dst[f] + (two_d ? b.sk2 : b.sk3 + b.layer * (k - 1));
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int r = ty; r < 32; r += 8) {
        const int j = jb + r, i = t0 + tx - j;
        double v = 0.0;
        if (j <= n1 && i >= 1 && i <= n0) v = s[(i - 1) + (long)n0 * (j - 1)];
        tile[r][tx] = v;
    }
    __syncthreads();
    for (int q = ty; q < 32; q += 8) {
        const int t = t0 + q, j = jb + tx, i = t - j;
        if (j <= n1 && i >= 1 && i <= n0) d[(long)(t - 2) * b.vp + (j - 1)] = (S)tile[tx][q];
    }
}

// The reverse for the swept scalar and its history, interior points only:
// the same (plane, row) tiles, read along j, written along i
template <typename S>
__global__ void __launch_bounds__(256) k_unskew(const SkewBlk *__restrict__ sb, const S *__restrict__ sks,
                                                const S *__restrict__ skh, double *__restrict__ sc1,
                                                double *__restrict__ hsc1, int ntp)
{
    __shared__ double tile[2][32][33];
    const SkewBlk b = sb[blockIdx.z];
    const int n0 = b.n[0], n1 = b.n[1];
    const int k = blockIdx.y + 2;
    if (k > b.n[2] - 1) return;
    const int tt = blockIdx.x % ntp, jt = blockIdx.x / ntp;
    if (jt * 32 >= n1 || 32 * tt > n0 + n1 - 2) return;
    const int t0 = 2 + 32 * tt, jb = 1 + 32 * jt;
    const long lay = b.sk3 + b.layer * (k - 1);
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int q = ty; q < 32; q += 8) {
        const int t = t0 + q, j = jb + tx, i = t - j;
        double a = 0.0, h = 0.0;
        if (j >= 2 && j <= n1 - 1 && i >= 2 && i <= n0 - 1) {
            const long e = lay + (long)(t - 2) * b.vp + (j - 1);
            a = (double)sks[e];
            h = (double)skh[e];
        }
        tile[0][tx][q] = a;
        tile[1][tx][q] = h;
    }
    __syncthreads();
    const long base = b.off3 + (long)n0 * n1 * (k - 1);
    for (int r = ty; r < 32; r += 8) {
        const int j = jb + r, i = t0 + tx - j;
        if (j >= 2 && j <= n1 - 1 && i >= 2 && i <= n0 - 1) {
            const long p = base + (i - 1) + (long)n0 * (j - 1);
            sc1[p] = tile[0][r][tx];
            hsc1[p] = tile[1][r][tx];
        }
    }
}

// the new-value array's initial state
template <typename S> __global__ void k_fill_sentinel(S *__restrict__ p, long n)
{
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        p[e] = (S)kSentinel;
}

// ----------------------------------------------------------- the pipeline
// R: arithmetic type; S: storage type of the skewed copies; FAST: the
// reciprocal tables of the fast builds; D: planes staged ahead.
//
// One CTA: three compute threads per row of the tile -- thread (d, r)
// computes the two faces of axis d of the row's point (gradients, limited
// face values, convective and diffusive fluxes), the x thread then adds
// the three axes' flux differences in the reference's order and updates
// the point -- and, last, one producer warp whose lanes stage the vectors
// of each plane with 16-byte cp.async copies, one cp.async group per plane
// step.  At plane step u the producer waits for its group u - (D-1); the
// __syncthreads that opens step u+1 then publishes it to the compute
// threads, which read group u+1-D there: D groups are in flight.
template <typename R, typename S, bool FAST, int D>
__global__ void __launch_bounds__(kSweepThreadsMax) k_sc1_tiles(SweepArgs<S> A, double dtime_d, long limit)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    S *ring = (S *)smem_raw;
    __shared__ int s_tile, s_ok[2];  // s_ok by plane parity: thread 0 may write the next before all read this
    __shared__ R part[4][kSweepRows];  // y and z flux differences of each row's point
    constexpr int E = 16 / sizeof(S);  // elements per 16-byte chunk
    const R lambda = (R)4.0, small = (R)1.e-30, half = (R)0.5, one = (R)1.0, zero = (R)0.0;
    const R dtime = (R)dtime_d;
    const int tid = threadIdx.x, lane = tid & 31;
    const int rpad = ((int)blockDim.x - 32) / 3;  // rows per axis group (a multiple of 32)
    const int ncomp = 3 * rpad;                    // compute threads
    const bool producer = tid >= ncomp;
    const int axis = producer ? 0 : tid / rpad, r = producer ? 0 : tid - axis * rpad;
    for (;;) {
        if (tid == 0) {
            int tk = -1;
            if (!*(volatile int *)A.err) tk = atomicAdd(A.ticket, 1);
            s_tile = tk;
        }
        __syncthreads();
        const int tix = s_tile;
        if (tix < 0 || tix >= A.ntile) return;
        const SweepTile T = A.tiles[tix];
        const SkewBlk b = A.sb[T.blk];
        const int n0 = b.n[0], n1 = b.n[1], n2 = b.n[2];
        const int k = T.k, j0 = T.j0, j1 = T.j1;
        const int ni = n0 - 1, nj = n1 - 1, nk = n2 - 1;
        const bool jhalo = T.up_j >= 0;  // rows j0-2, j0-1 belong to another tile
        // staged rows: j0-2 .. j1+1 (0-based jr), chunk aligned
        const int sbase = (max(0, j0 - 3) / E) * E;
        const int jr_lo = max(0, j0 - 3), jr_hi = min(n1, j1 + 1);  // [lo, hi)
        const int SW = A.sw;
        // own row and the plane range
        const int j = j0 + r;
        const bool row = !producer && j < j1;
        const int t0 = 2 + j0, t1 = ni + (j1 - 1);
        const int ts = t0 - D - 4;
        // 1-D metrics of this layer
        const double *dkp = A.dkp + b.off1k, *dkw = A.dkw + b.off1k;
        const R dkw_k = (R)dkw[k - 1];
        const R dkp_m3 = k > 2 ? (R)dkp[k - 3] : zero, dkp_m2 = (R)dkp[k - 2], dkp_m1 = (R)dkp[k - 1];
        const R dkp_0 = k < nk ? (R)dkp[k] : zero;
        R rdkp_m3 = zero, rdkp_m2 = zero, rdkp_m1 = zero, rdkp_0 = zero;
        if (FAST) {
            const double *rdkp = A.rdkp + b.off1k;
            rdkp_m3 = k > 2 ? (R)rdkp[k - 3] : zero;
            rdkp_m2 = (R)rdkp[k - 2];
            rdkp_m1 = (R)rdkp[k - 1];
            rdkp_0 = k < nk ? (R)rdkp[k] : zero;
        }
        // ring element of vector v, plane p, row jj
        const int rowoff = j - 1 - sbase;
        auto slot = [&](int v, int p, int jj) -> S & {
            return ring[(vprefix(FAST, v, D) + (p & (vslots(v, D) - 1))) * SW + rowoff + (jj - j)];
        };
        auto at = [&](int v, int p, int jj) -> R { return (R)slot(v, p, jj); };
        // element (plane p, row jj) of layer kv in a skewed 3-D array
        auto e3 = [&](int kv, int p, int jj) -> long {
            return b.sk3 + b.layer * (kv - 1) + (long)(p - 2) * b.vp + (jj - 1);
        };
        // a new value of layer kv at (p, jj), staged in vector v
        auto newval = [&](int v, int kv, int p, int jj) -> R {
            return (R)fresh<S>(slot(v, p, jj), A.scnew + e3(kv, p, jj), A.err, limit);
        };
        // producer: the copies of group t, plane t + D + hi of every vector,
        // chunks spread over the lanes
        auto issue = [&](int t) {
#pragma unroll
            for (int v = 0; v < V_N; v++) {
                if (!has_vec(FAST, v)) continue;
                const VecDesc vd = vdesc(v);
                const int p = t + D + vd.hi;
                if (p < t0 + vd.lo || p > t1 + vd.hi || p < 2 || p > n0 + n1) continue;
                const int kv = k + vd.dk;
                if (kv < 1 || kv > n2) continue;
                if (v == V_SCH && !jhalo) continue;
                const bool cross = vd.dk != 0;
                int lo = cross ? j0 - 1 : v == V_SCH ? max(0, j0 - 3) : jr_lo;
                int hi = cross ? j1 - 1 : v == V_SCH ? j0 - 1 : jr_hi;
                lo = max(lo, p - n0 - 1);
                hi = min(hi, p - 1);
                if (lo >= hi) continue;
                const int c_lo = lo / E, c_hi = (hi + E - 1) / E;
                const S *g;
                if (vd.src < 8) {
                    // new values of an interior layer below from the new-value array
                    const bool nw = vd.src == 0 && vd.dk < 0 && kv >= 2 && kv <= n2 - 1;
                    g = (nw ? A.scnew : A.f3[vd.src]) + b.sk3 + b.layer * (kv - 1) + (long)(p - 2) * b.vp;
                } else if (vd.src < 18) {
                    g = A.f2[vd.src - 8] + b.sk2 + (long)(p - 2) * b.vp;
                } else {
                    g = A.scnew + b.sk3 + b.layer * (kv - 1) + (long)(p - 2) * b.vp;
                }
                S *dst = ring + (vprefix(FAST, v, D) + (p & (vslots(v, D) - 1))) * SW - sbase;
                for (int c = c_lo + lane; c < c_hi; c += 32) cp_async16(dst + c * E, g + c * E);
            }
        };
        bool ok = true;
        int t = ts;
        int err_seen = 0;  // thread 0: the error flag, re-read from L2 every 16 planes only
        for (; t <= t1; t++) {
            if (tid == 0) {
                if (((t - ts) & 15) == 0) err_seen = *(volatile int *)A.err;
                s_ok[t & 1] = !err_seen;
            }
            __syncthreads();
            if (!s_ok[t & 1]) {
                ok = false;
                break;
            }
            if (producer) {
                issue(t);
                cp_async_commit();
                cp_async_wait<D - 1>();
                continue;
            }
            const int i = t - j;
            const bool pt = t >= t0 && row && i >= 2 && i <= ni;
            // ---- one point of set_sc1_block.F:104-502 (sc1_cell's operands),
            // axis by axis
            R c_d = zero, t_d = zero;  // this axis: g_hi - g_lo and t_hi - t_lo
            if (pt) {
                const R s0 = at(V_SC, t, j);
                const R rho0 = at(V_RHO, t, j), gs0 = at(V_GS, t, j), gl0 = at(V_GL, t, j);
                const long gst = A.gstride;
                const int gm = A.gm;
                const double *GR = A.grad;
                const int bi = T.blk;
                R rlo, rhi, gslo, gshi, gllo, glhi, vlo, vhi, slo, shi, dlo, dmid, dhi;  // faces' operands
                R areal, areah, glo_m, ghi_p;  // face areas; gradient beyond each face
                int s_lo, s_hi;                // sides of the two faces
                bool first, last;              // the point is the first / last interior one along the axis
                if (axis == 0) {
                    rlo = at(V_RHO, t - 1, j); rhi = at(V_RHO, t + 1, j);
                    gslo = at(V_GS, t - 1, j); gshi = at(V_GS, t + 1, j);
                    gllo = at(V_GL, t - 1, j); glhi = at(V_GL, t + 1, j);
                    vlo = at(V_U, t, j); vhi = at(V_U, t + 1, j);
                    slo = at(V_SC, t - 1, j); shi = at(V_SC, t + 1, j);
#define QD(x, v, vr, pp, jj) (FAST ? (x) * at(vr, pp, jj) : (x) / at(v, pp, jj))
                    dlo = QD(s0 - slo, V_DIU, V_RDIU, t, j);
                    dhi = QD(shi - s0, V_DIU, V_RDIU, t + 1, j);
                    first = i == 2;
                    last = i == ni;
                    s_lo = 0;
                    s_hi = 1;
                    glo_m = first ? ((b.bc[0] != LES_BCT_INTERFACE_D) ? dlo
                                     : (R)GR[(long)(A.link[bi * 6 + 0]) * 6 * gst + 1 * gst + (j - 1) + (long)gm * (k - 1)])
                                  : QD(slo - at(V_SC, t - 2, j), V_DIU, V_RDIU, t - 1, j);
                    ghi_p = last ? ((b.bc[1] != LES_BCT_INTERFACE_D) ? dhi
                                    : (R)GR[(long)(A.link[bi * 6 + 1]) * 6 * gst + 0 * gst + (j - 1) + (long)gm * (k - 1)])
                                 : QD(at(V_SC, t + 2, j) - shi, V_DIU, V_RDIU, t + 2, j);
                    areal = at(V_RDJU, t, j) * dkw_k;
                    areah = at(V_RDJU, t + 1, j) * dkw_k;
                } else if (axis == 1) {
                    rlo = at(V_RHO, t - 1, j - 1); rhi = at(V_RHO, t + 1, j + 1);
                    gslo = at(V_GS, t - 1, j - 1); gshi = at(V_GS, t + 1, j + 1);
                    gllo = at(V_GL, t - 1, j - 1); glhi = at(V_GL, t + 1, j + 1);
                    vlo = at(V_V, t, j); vhi = at(V_V, t + 1, j + 1);
                    slo = (jhalo && j == j0) ? newval(V_SCH, k, t - 1, j - 1) : at(V_SC, t - 1, j - 1);
                    shi = at(V_SC, t + 1, j + 1);
                    dlo = QD(s0 - slo, V_DJV, V_RDJV, t, j);
                    dhi = QD(shi - s0, V_DJV, V_RDJV, t + 1, j + 1);
                    first = j == 2;
                    last = j == nj;
                    glo_m = first ? ((b.bc[2] != LES_BCT_INTERFACE_D) ? dlo
                                     : (R)GR[(long)(A.link[bi * 6 + 2]) * 6 * gst + 3 * gst + (i - 1) + (long)gm * (k - 1)])
                                  : QD(slo - ((jhalo && j - 2 < j0) ? newval(V_SCH, k, t - 2, j - 2) : at(V_SC, t - 2, j - 2)),
                                       V_DJV, V_RDJV, t - 1, j - 1);
                    ghi_p = last ? ((b.bc[3] != LES_BCT_INTERFACE_D) ? dhi
                                    : (R)GR[(long)(A.link[bi * 6 + 3]) * 6 * gst + 2 * gst + (i - 1) + (long)gm * (k - 1)])
                                 : QD(at(V_SC, t + 2, j + 2) - shi, V_DJV, V_RDJV, t + 2, j + 2);
#undef QD
                    areal = at(V_RDIV, t, j) * dkw_k;
                    areah = at(V_RDIV, t + 1, j + 1) * dkw_k;
                    s_lo = 2;
                    s_hi = 3;
                } else {
                    rlo = at(V_RHOM1, t, j); rhi = at(V_RHOP1, t, j);
                    gslo = at(V_GSM1, t, j); gshi = at(V_GSP1, t, j);
                    gllo = at(V_GLM1, t, j); glhi = at(V_GLP1, t, j);
                    vlo = at(V_W, t, j); vhi = at(V_WP1, t, j);
                    slo = k - 1 >= 2 ? newval(V_SCM1, k - 1, t, j) : at(V_SCM1, t, j);
                    shi = at(V_SCP1, t, j);
                    const R rpij = at(V_RP, t, j);
                    const R rrpij = FAST ? at(V_RRP, t, j) : zero;
#define QZ(x, dk_, rdk_) (FAST ? (x) * (rrpij * (rdk_)) : (x) / (rpij * (dk_)))
                    dlo = QZ(s0 - slo, dkp_m2, rdkp_m2);
                    dhi = QZ(shi - s0, dkp_m1, rdkp_m1);
                    first = k == 2;
                    last = k == nk;
                    glo_m = first ? ((b.bc[4] != LES_BCT_INTERFACE_D) ? dlo
                                     : (R)GR[(long)(A.link[bi * 6 + 4]) * 6 * gst + 5 * gst + (i - 1) + (long)gm * (j - 1)])
                                  : QZ(slo - (k - 2 >= 2 ? newval(V_SCM2, k - 2, t, j) : at(V_SCM2, t, j)), dkp_m3, rdkp_m3);
                    ghi_p = last ? ((b.bc[5] != LES_BCT_INTERFACE_D) ? dhi
                                    : (R)GR[(long)(A.link[bi * 6 + 5]) * 6 * gst + 4 * gst + (i - 1) + (long)gm * (j - 1)])
                                 : QZ(at(V_SCP2, t, j) - shi, dkp_0, rdkp_0);
#undef QZ
                    areal = at(V_DIDJP, t, j);
                    areah = areal;
                    s_lo = 4;
                    s_hi = 5;
                }
                (void)s_lo;
                (void)s_hi;
                (void)dmid;
                const R rholf = half * (rho0 + rlo);
                const R rhohf = half * (rho0 + rhi);
                const R gamlf = half * (gs0 + gslo) * rholf + half * (gl0 + gllo);
                const R gamhf = half * (gs0 + gshi) * rhohf + half * (gl0 + glhi);
                // low face tests v >= 0, high face v > 0 (rwst / rest of the reference)
                const R rl = (vlo >= zero) ? (glo_m + small) / (dlo + small) : (dhi + small) / (dlo + small);
                const R rh = (vhi > zero) ? (dlo + small) / (dhi + small) : (ghi_p + small) / (dhi + small);
                const R liml = fmax(zero, fmin(lambda * rl, one));
                const R limh = fmax(zero, fmin(lambda * rh, one));
                R fl, fh;
                if (vlo > zero) fl = slo + half * liml * (s0 - slo);
                else if (vlo < zero) fl = s0 + half * liml * (slo - s0);
                else fl = half * (s0 + slo);
                if (vhi > zero) fh = s0 + half * limh * (shi - s0);
                else if (vhi < zero) fh = shi + half * limh * (s0 - shi);
                else fh = half * (s0 + shi);
                const R gl_ = rholf * vlo * fl * areal;
                const R gh_ = rhohf * vhi * fh * areah;
                const R tl_ = gamlf * areal * dlo;
                const R th_ = gamhf * areah * dhi;
                c_d = gh_ - gl_;
                t_d = th_ - tl_;
                if (axis > 0) {
                    part[2 * (axis - 1)][r] = c_d;
                    part[2 * (axis - 1) + 1][r] = t_d;
                }
            }
            asm volatile("bar.sync 1, %0;" ::"r"(ncomp) : "memory");  // the compute threads
            if (pt && axis == 0) {
                // combine in the reference's order:
                // convf = -(gef - gwf) - (gnf - gsf) - (grf - glf), difff likewise
                const R convf = -c_d - part[0][r] - part[2][r];
                const R difff = (t_d + part[1][r]) + part[3][r];
                const R h = convf + difff;
                const R s0 = at(V_SC, t, j);
                const R vol = at(V_RDIDJP, t, j) * dkw_k;
                R tmp = s0 + dtime / (vol * at(V_RHO, t, j)) * ((R)1.5 * h - half * at(V_H, t, j));
                if (tmp < zero) tmp = zero;
                if (tmp > one) tmp = one;
                // the new value: in the ring slot of plane t (read by later
                // planes of this tile) and in the new-value array (read by the
                // layers above and the tile above); the history in place
                slot(V_SC, t, j) = (S)tmp;
                const long e = e3(k, t, j);
                st_strong(A.scnew + e, (S)tmp);
                A.f3[1][e] = (S)h;
            }
        }
        // the copies still in flight land before the ring is reused or the
        // CTA exits
        if (producer) cp_async_wait_all();
        __syncthreads();
        if (!ok) return;
    }
}

} // namespace
} // namespace les_sweep

namespace SWEEP_NS {

using namespace les_sweep;

template <typename S>
void launch_skew_t(const SkewBlk *sb, int nb, int maxn0, int maxn1, int maxn2, int nfield,
                   const SkewPtrs<S> &P, int two_d, cudaStream_t st)
{
    const int ntp = (maxn0 + maxn1 - 1 + 31) / 32, njt = (maxn1 + 31) / 32;
    k_skew<S><<<dim3(ntp * njt, two_d ? 1 : maxn2, nb * nfield), 256, 0, st>>>(sb, nfield, P, two_d, ntp);
    les::count_launch(1);
}

template <typename S>
void launch_unskew_t(const SkewBlk *sb, int nb, int maxn0, int maxn1, int maxn2, const S *sks, const S *skh,
                     double *sc1, double *hsc1, cudaStream_t st)
{
    const int ntp = (maxn0 + maxn1 - 1 + 31) / 32, njt = (maxn1 + 31) / 32;
    k_unskew<S><<<dim3(ntp * njt, maxn2 > 2 ? maxn2 - 2 : 1, nb), 256, 0, st>>>(sb, sks, skh, sc1, hsc1, ntp);
    les::count_launch(1);
}

template <typename S> void launch_fill_t(S *p, long n, cudaStream_t st)
{
    long g = (n + 255) / 256;
    k_fill_sentinel<S><<<(unsigned)(g > 8192 ? 8192 : g), 256, 0, st>>>(p, n);
    les::count_launch(1);
}

template <typename R, typename S, bool FAST, int D>
int tiles_smem(int sw)
{
    return ring_slots(FAST, D) * sw * (int)sizeof(S);
}

template <typename R, typename S, bool FAST, int D>
cudaError_t launch_tiles_t(const SweepArgs<S> &a, double dtime, long limit, int nctas, int nthr, cudaStream_t st)
{
    const int smem = tiles_smem<R, S, FAST, D>(a.sw);
    auto kern = k_sc1_tiles<R, S, FAST, D>;
    kern<<<nctas, nthr, smem, st>>>(a, dtime, limit);
    les::count_launch(1);
    return cudaGetLastError();
}

// resident CTAs of nthr threads with the ring for row width sw (sets the
// kernel's dynamic shared-memory limit; called before any launch)
template <typename R, typename S, bool FAST, int D>
int tiles_max_ctas(int sw, int nthr)
{
    const int smem = tiles_smem<R, S, FAST, D>(sw);
    auto kern = k_sc1_tiles<R, S, FAST, D>;
    int dev = 0, nsm = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, nthr, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return nsm * per;
}

#if defined(LES_SWEEP_EXACT)
// FP64, the reference's operation order (this unit is built with -fmad=false)
using RT = double;
using ST = double;
constexpr bool kFast = false;
#else
// fast FP64 build: reciprocal tables and FMA contraction
using RT = double;
using ST = double;
constexpr bool kFast = true;
#endif

void launch_sweep_skew(const SkewBlk *sb, int nb, int maxn0, int maxn1, int maxn2, int nfield,
                       const SkewPtrs<double> &P, int two_d, cudaStream_t st)
{
    launch_skew_t<ST>(sb, nb, maxn0, maxn1, maxn2, nfield, P, two_d, st);
}
void launch_sweep_unskew(const SkewBlk *sb, int nb, int maxn0, int maxn1, int maxn2, const double *sks,
                         const double *skh, double *sc1, double *hsc1, cudaStream_t st)
{
    launch_unskew_t<ST>(sb, nb, maxn0, maxn1, maxn2, sks, skh, sc1, hsc1, st);
}
void launch_sweep_fill(double *p, long n, cudaStream_t st) { launch_fill_t<ST>(p, n, st); }
int sweep_tiles_smem(int sw) { return tiles_smem<RT, ST, kFast, kSweepDepth>(sw); }
int sweep_tiles_max_ctas(int sw, int nthr) { return tiles_max_ctas<RT, ST, kFast, kSweepDepth>(sw, nthr); }
cudaError_t launch_sweep_tiles(const SweepArgs<double> &a, double dtime, long limit, int nctas, int nthr,
                               cudaStream_t st)
{
    return launch_tiles_t<RT, ST, kFast, kSweepDepth>(a, dtime, limit, nctas, nthr, st);
}

} // namespace SWEEP_NS

#if !defined(LES_SWEEP_EXACT)
// the FP32 build: FP32 arithmetic on FP32 skewed copies
namespace les_f32 {
using namespace les_sweep;
void launch_sweep_skew(const SkewBlk *sb, int nb, int maxn0, int maxn1, int maxn2, int nfield,
                       const SkewPtrs<float> &P, int two_d, cudaStream_t st)
{
    les_fast::launch_skew_t<float>(sb, nb, maxn0, maxn1, maxn2, nfield, P, two_d, st);
}
void launch_sweep_unskew(const SkewBlk *sb, int nb, int maxn0, int maxn1, int maxn2, const float *sks,
                         const float *skh, double *sc1, double *hsc1, cudaStream_t st)
{
    les_fast::launch_unskew_t<float>(sb, nb, maxn0, maxn1, maxn2, sks, skh, sc1, hsc1, st);
}
void launch_sweep_fill(float *p, long n, cudaStream_t st) { les_fast::launch_fill_t<float>(p, n, st); }
int sweep_tiles_smem(int sw) { return les_fast::tiles_smem<float, float, true, kSweepDepth>(sw); }
int sweep_tiles_max_ctas(int sw, int nthr) { return les_fast::tiles_max_ctas<float, float, true, kSweepDepth>(sw, nthr); }
cudaError_t launch_sweep_tiles(const SweepArgs<float> &a, double dtime, long limit, int nctas, int nthr,
                               cudaStream_t st)
{
    return les_fast::launch_tiles_t<float, float, true, kSweepDepth>(a, dtime, limit, nctas, nthr, st);
}
} // namespace les_f32
#endif
