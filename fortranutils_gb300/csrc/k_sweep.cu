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
//    plane t of a layer is one contiguous vector over j and the fields of a
//    block follow one another at a fixed stride, so (rows, planes, fields)
//    is a 3-D tensor: one TMA tensor copy stages the plane vectors of
//    several fields of a layer into a shared-memory ring, D planes ahead
//    (eight copies per plane: the layer's own fields, those of the layers
//    k-1, k-2, k+1, k+2 it reads, the 2-D metric tables, the new values of
//    the tile below); the new values go to the new-value array and to the
//    ring (read by later planes of the tile) and are copied to the FP64
//    fields at the end (k_unskew).
//
// The arithmetic per point is that of sc1_cell in k_phys.cu, operand for
// operand, so the exact build (FP64, -fmad=false) equals the hyperplane
// sweep and the oracle bit for bit; the fast build uses the reciprocal
// metric tables (x * (1/d)) as k_phys.cu's fast build does; the FP32 build
// is the same template with R = S = float (FP64 fields in HBM, FP32 skewed
// copies).
#include <cuda.h>

#include "k_common.cuh"
#include "kernels.h"

#if defined(LES_SWEEP_EXACT)
#define SWEEP_NS les_exact
#else
#define SWEEP_NS les_fast
#endif

namespace les_sweep {
namespace {  // internal to each build of this unit

// Copy groups staged per plane.  Fields of the skewed 3-D tensor: 0 sc1
// (old values), 1 hsc1, 2 u, 3 v, 4 w, 5 rho, 6 gamsc1, 7 gamlam, 8 the new
// values of sc1 (sentinel until computed; old values on ghost points).
// Per group: layer offset, first field, fields, the plane window
// [t+lo, t+hi] a point of plane t reads, and the tensor map it copies with
// (0: 8 fields, 1: 4 fields, 2: 1 field, 3: the 2-D tables).
enum { GR_OWN, GR_M1, GR_M2, GR_P1A, GR_P1B, GR_P2, GR_SCH, GR_2D, GR_N };
struct GroupDesc {
    int dk, f0, nf, lo, hi, map;
};
__host__ __device__ constexpr GroupDesc gdesc(int g, bool fast)
{
    return g == GR_OWN ? GroupDesc{0, 0, 8, -2, 2, 0}
           : g == GR_M1 ? GroupDesc{-1, 5, 4, 0, 0, 1}   // rho gamsc1 gamlam new sc1 of k-1
           : g == GR_M2 ? GroupDesc{-2, 8, 1, 0, 0, 2}   // new sc1 of k-2
           : g == GR_P1A ? GroupDesc{1, 4, 4, 0, 0, 1}   // w rho gamsc1 gamlam of k+1
           : g == GR_P1B ? GroupDesc{1, 0, 1, 0, 0, 2}   // old sc1 of k+1
           : g == GR_P2 ? GroupDesc{2, 0, 1, 0, 0, 2}    // old sc1 of k+2
           : g == GR_SCH ? GroupDesc{0, 8, 1, -2, -1, 2} // new sc1, rows of the tile below
                         : GroupDesc{0, 0, fast ? 10 : 7, -1, 2, 3};
}
// 2-D tables: diu djv rdju rdiv rp didjp rdidjp (1/diu 1/djv 1/rp)
enum { T_DIU, T_DJV, T_RDJU, T_RDIV, T_RP, T_DIDJP, T_RDIDJP, T_RDIU, T_RDJV, T_RRP };

__host__ __device__ constexpr int pow2_ceil(int n) { return n <= 1 ? 1 : 2 * pow2_ceil((n + 1) / 2); }
// ring slots of group g: planes t+lo .. t+hi+D, a power of two (slot of
// plane p = p & (slots-1))
__host__ __device__ constexpr int gslots(int g, bool fast, int D)
{
    return pow2_ceil(gdesc(g, fast).hi - gdesc(g, fast).lo + D + 1);
}
// elements of one slot of group g for ring row width sw, rounded up to 128
// bytes (the alignment of a tensor copy's destination)
__host__ __device__ constexpr int gslot_elems(int g, bool fast, int sw, int esz)
{
    return (gdesc(g, fast).nf * sw * esz + 127) / 128 * 128 / esz;
}
// ring elements before group g
__host__ __device__ constexpr int gbase(int g, bool fast, int D, int sw, int esz)
{
    int s = 0;
    for (int q = 0; q < g; q++) s += gslots(q, fast, D) * gslot_elems(q, fast, sw, esz);
    return s;
}

// the new-value array's initial value on interior points: the scalar is
// clamped to [0, 1]
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
__device__ __forceinline__ void mbar_init(unsigned long long *m, int count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(m)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned long long *m, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(m)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned long long *m, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(smem_addr(m)), "r"(parity)
                 : "memory");
    return ok != 0;
}
// one box of a 3-D tensor map (global memory) into shared memory by the TMA
// unit, completing its bytes on the mbarrier
__device__ __forceinline__ void tensor_copy(void *dst, const void *map, int x, int y, int z, unsigned long long *m)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_addr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(m))
        : "memory");
}
// wait for a phase of an mbarrier; bounded: after `limit` tries, or once
// another CTA has set *err, give up (sets *err)
__device__ __forceinline__ bool mbar_wait(unsigned long long *m, unsigned parity, int *err, long limit)
{
    long it = 0;
    while (!mbar_try(m, parity)) {
        if (++it > limit || *(volatile int *)err) {
            atomicExch(err, 1);
            return false;
        }
    }
    return true;
}
// the same for the copies in flight when a tile ends, even after an error
// elsewhere (they depend on nothing); bounded
__device__ __forceinline__ void mbar_drain(unsigned long long *m, unsigned parity, int *err, long limit)
{
    long it = 0;
    while (!mbar_try(m, parity))
        if (++it > limit) {
            atomicExch(err, 1);
            return;
        }
}

// A new value staged from the new-value array: while it is still the
// sentinel, re-read it from L2 (another CTA is computing it); bounded by
// `limit` polls, or until another CTA has set *err (then *err is set and
// the staged value returned: the call reports LES_ERR_TIMEOUT).
// The error flag is read every 64 polls only (each read is an L2 round
// trip of its own).
template <typename S>
__device__ S fresh(S v, const S *g, int *err, long limit)
{
    long it = 0;
    while (v == (S)kSentinel) {
        if ((++it & 63) == 0) {
            if (*(volatile int *)err) return v;
            if (it > limit) {
                atomicExch(err, 1);
                return v;
            }
        }
        if (it > 4) __nanosleep(32);
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

// The new-value array's initial state: the sentinel on interior points,
// the old scalar (field 0) on ghost points, which no tile changes
template <typename S>
__global__ void __launch_bounds__(256) k_init_new(const SkewBlk *__restrict__ sb, const S *__restrict__ old,
                                                  S *__restrict__ nw)
{
    const SkewBlk b = sb[blockIdx.y];
    const long n = b.layer * b.n[2];
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const long kv = e / b.layer, rem = e - kv * b.layer;
        const int p = (int)(rem / b.vp) + 2, jr = (int)(rem - (long)(p - 2) * b.vp);
        const int i = p - (jr + 1), j = jr + 1, k = (int)kv + 1;
        const bool inner = i >= 2 && i <= b.n[0] - 1 && j >= 2 && j <= b.n[1] - 1 && k >= 2 && k <= b.n[2] - 1;
        nw[b.sk3 + e] = inner ? (S)kSentinel : old[b.sk3 + e];
    }
}

// ----------------------------------------------------------- the pipeline
// R: arithmetic type; S: storage type of the skewed copies; FAST: the
// reciprocal tables of the fast builds; D: planes staged ahead.
// One CTA: compute warps (one thread per row of the tile) and, last, one
// producer warp whose lane g issues the tensor copy of group g for each
// plane.  Plane group u (the copies issued at the u-th plane step of the
// CTA) completes mbarrier u % (D+1); warp 0 waits for group u - D before
// plane step u and the __syncthreads that follows publishes it, so D
// groups are in flight.
template <typename R, typename S, bool FAST, int D>
__global__ void __launch_bounds__(kSweepThreads + 32) k_sc1_tiles(SweepArgs<S> A, double dtime_d, long limit)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    S *ring = (S *)smem_raw;
    constexpr int G = D + 1;
    __shared__ __align__(8) unsigned long long mbar[G];
    __shared__ int s_tile, s_ok[2];  // s_ok by plane parity: thread 0 may write the next before all read this
    constexpr int E = 16 / sizeof(S);  // elements per 16-byte chunk
    constexpr int ESZ = sizeof(S);
    const R lambda = (R)4.0, small = (R)1.e-30, half = (R)0.5, one = (R)1.0, zero = (R)0.0;
    const R dtime = (R)dtime_d;
    const int tid = threadIdx.x, lane = tid & 31;
    const int nwc = (int)(blockDim.x >> 5) - 1;  // compute warps
    const bool producer = (tid >> 5) == nwc;
    const int SW = A.sw;
    if (tid == 0)
        for (int g = 0; g < G; g++) mbar_init(&mbar[g], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();
    long ubase = 0;  // plane steps of earlier tiles (mbarrier phases continue)
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
        const int np = n0 + n1 - 1;      // planes of a layer
        const bool jhalo = T.up_j >= 0;  // rows j0-2, j0-1 belong to another tile
        const int sbase = (max(0, j0 - 3) / E) * E;  // first staged row (0-based), 16-byte aligned
        const int j = j0 + tid;
        const bool row = !producer && j < j1;
        const int t0 = 2 + j0, t1 = ni + (j1 - 1);
        const int ts = t0 - D - 4;
        // producer lane g: group g's fixed parts
        GroupDesc pg{0, 0, 0, 0, 0, 0};
        bool pg_on = false;
        const CUtensorMap *pg_map = nullptr;
        unsigned pg_bytes = 0;
        S *pg_ring = nullptr;
        int pg_slots = 1, pg_slot_elems = 0;
        if (producer && lane < GR_N) {
            pg = gdesc(lane, FAST);
            const int kv = k + pg.dk;
            pg_on = kv >= 1 && kv <= n2 && (lane != GR_SCH || jhalo);
            pg_map = (const CUtensorMap *)A.tmaps + 4 * T.blk + pg.map;
            pg_bytes = (unsigned)(pg.nf * SW * ESZ);
            pg_slots = pow2_ceil(pg.hi - pg.lo + D + 1);
            pg_slot_elems = (pg.nf * SW * ESZ + 127) / 128 * 128 / ESZ;
            int base = 0;
            for (int q = 0; q < lane; q++) base += gslots(q, FAST, D) * gslot_elems(q, FAST, SW, ESZ);
            pg_ring = ring + base;
        }
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
        // ring element of group g, field fl, plane p, row jj
        const int rowoff = j - 1 - sbase;
        auto slot = [&](int g, int fl, int p, int jj) -> S & {
            return ring[gbase(g, FAST, D, SW, ESZ) + (p & (gslots(g, FAST, D) - 1)) * gslot_elems(g, FAST, SW, ESZ) +
                        fl * SW + rowoff + (jj - j)];
        };
        auto at = [&](int g, int fl, int p, int jj) -> R { return (R)slot(g, fl, p, jj); };
        // element (plane p, row jj) of layer kv in a skewed 3-D array
        auto e3 = [&](int kv, int p, int jj) -> long {
            return b.sk3 + b.layer * (kv - 1) + (long)(p - 2) * b.vp + (jj - 1);
        };
        // a new value of layer kv at (p, jj), staged in group g, field fl
        auto newval = [&](int g, int fl, int kv, int p, int jj) -> R {
            return (R)fresh<S>(slot(g, fl, p, jj), A.scnew + e3(kv, p, jj), A.err, limit);
        };
#define SC(p, jj) at(GR_OWN, 0, p, jj)
#define TB(tb, p, jj) at(GR_2D, tb, p, jj)
        bool ok = true;
        int t = ts;
        int err_seen = 0;
  // thread 0: the error flag, re-read from L2 every 16 planes only
        for (; t <= t1; t++) {
            const long u = ubase + (t - ts);
            if (tid == 0) {
                if (((t - ts) & 15) == 0) err_seen = *(volatile int *)A.err;
                s_ok[t & 1] = !err_seen;
            }
            if (tid < 32 && u >= D) mbar_wait(&mbar[(u - D) % G], (unsigned)(((u - D) / G) & 1), A.err, limit);
            __syncthreads();
            if (!s_ok[t & 1]) {
                ok = false;
                break;
            }
            if (producer) {
                // group u: plane t + D + hi of every copy group
                const int p = t + D + pg.hi;
                const bool go = pg_on && p >= t0 + pg.lo && p <= t1 + pg.hi && p >= 2 && p <= n0 + n1;
                const unsigned total = __reduce_add_sync(0xffffffffu, go ? pg_bytes : 0u);
                if (lane == 0) mbar_expect(&mbar[u % G], total);
                __syncwarp();
                if (go) {
                    const int y = pg.map == 3 ? p - 2 : (k + pg.dk - 1) * np + (p - 2);
                    tensor_copy(pg_ring + (p & (pg_slots - 1)) * pg_slot_elems, pg_map, sbase, y, pg.f0, &mbar[u % G]);
                }
                continue;
            }
            if (t < t0 || !row) continue;
            const int i = t - j;
            if (i < 2 || i > ni) continue;
            // the new values of the two layers below: staged, or still the
            // sentinel when staged; then their L2 re-reads are issued here,
            // first, and overlap the rest of the point's work
            S m1 = slot(GR_M1, 3, t, j), m2 = k != 2 ? slot(GR_M2, 0, t, j) : (S)0;
            if (m1 == (S)kSentinel) m1 = ld_strong(A.scnew + e3(k - 1, t, j));
            if (m2 == (S)kSentinel) m2 = ld_strong(A.scnew + e3(k - 2, t, j));
            // ---- one point of set_sc1_block.F:104-502 (sc1_cell's operands)
            const R rho0 = at(GR_OWN, 5, t, j);
            const R rhowf = half * (rho0 + at(GR_OWN, 5, t - 1, j));
            const R rhoef = half * (rho0 + at(GR_OWN, 5, t + 1, j));
            const R rhosf = half * (rho0 + at(GR_OWN, 5, t - 1, j - 1));
            const R rhonf = half * (rho0 + at(GR_OWN, 5, t + 1, j + 1));
            const R rholf = half * (rho0 + at(GR_M1, 0, t, j));
            const R rhorf = half * (rho0 + at(GR_P1A, 1, t, j));
            const R rhop = rho0;
            const R gs0 = at(GR_OWN, 6, t, j), gl0 = at(GR_OWN, 7, t, j);
            const R gamwf = half * (gs0 + at(GR_OWN, 6, t - 1, j)) * rhowf + half * (gl0 + at(GR_OWN, 7, t - 1, j));
            const R gamef = half * (gs0 + at(GR_OWN, 6, t + 1, j)) * rhoef + half * (gl0 + at(GR_OWN, 7, t + 1, j));
            const R gamsf = half * (gs0 + at(GR_OWN, 6, t - 1, j - 1)) * rhosf + half * (gl0 + at(GR_OWN, 7, t - 1, j - 1));
            const R gamnf = half * (gs0 + at(GR_OWN, 6, t + 1, j + 1)) * rhonf + half * (gl0 + at(GR_OWN, 7, t + 1, j + 1));
            const R gamlf = half * (gs0 + at(GR_M1, 1, t, j)) * rholf + half * (gl0 + at(GR_M1, 2, t, j));
            const R gamrf = half * (gs0 + at(GR_P1A, 2, t, j)) * rhorf + half * (gl0 + at(GR_P1A, 3, t, j));
            const R uwf = at(GR_OWN, 2, t, j), uef = at(GR_OWN, 2, t + 1, j);
            const R vsf = at(GR_OWN, 3, t, j), vnf = at(GR_OWN, 3, t + 1, j + 1);
            const R wlf = at(GR_OWN, 4, t, j), wrf = at(GR_P1A, 0, t, j);
            const R s0 = SC(t, j);
            const R sw = SC(t - 1, j), se = SC(t + 1, j);
            const R ss = (jhalo && j == j0) ? newval(GR_SCH, 0, k, t - 1, j - 1) : SC(t - 1, j - 1);
            const R sn = SC(t + 1, j + 1);
            // the layer below: new values (interior), old ones on its ghost layer
            const R sl = (R)fresh<S>(m1, A.scnew + e3(k - 1, t, j), A.err, limit);
            const R sr = at(GR_P1B, 0, t, j);
#define QD(x, tb, rtb, pp, jj) (FAST ? (x) * TB(rtb, pp, jj) : (x) / TB(tb, pp, jj))
            const R dfdxwf = QD(s0 - sw, T_DIU, T_RDIU, t, j);
            const R dfdxef = QD(se - s0, T_DIU, T_RDIU, t + 1, j);
            const long gst = A.gstride;
            const int gm = A.gm;
            const double *GR = A.grad;
            const int bi = T.blk;
            R dfdxwwf, dfdxeef, dfdyssf, dfdynnf, dfdzllf, dfdzrrf;
            if (i == 2)
                dfdxwwf = (b.bc[0] != LES_BCT_INTERFACE_D)
                              ? dfdxwf
                              : (R)GR[(long)(A.link[bi * 6 + 0]) * 6 * gst + 1 * gst + (j - 1) + (long)gm * (k - 1)];
            else
                dfdxwwf = QD(sw - SC(t - 2, j), T_DIU, T_RDIU, t - 1, j);
            if (i == ni)
                dfdxeef = (b.bc[1] != LES_BCT_INTERFACE_D)
                              ? dfdxef
                              : (R)GR[(long)(A.link[bi * 6 + 1]) * 6 * gst + 0 * gst + (j - 1) + (long)gm * (k - 1)];
            else
                dfdxeef = QD(SC(t + 2, j) - se, T_DIU, T_RDIU, t + 2, j);
            const R dfdysf = QD(s0 - ss, T_DJV, T_RDJV, t, j);
            const R dfdynf = QD(sn - s0, T_DJV, T_RDJV, t + 1, j + 1);
            if (j == 2)
                dfdyssf = (b.bc[2] != LES_BCT_INTERFACE_D)
                              ? dfdysf
                              : (R)GR[(long)(A.link[bi * 6 + 2]) * 6 * gst + 3 * gst + (i - 1) + (long)gm * (k - 1)];
            else
                dfdyssf = QD(ss - ((jhalo && j - 2 < j0) ? newval(GR_SCH, 0, k, t - 2, j - 2) : SC(t - 2, j - 2)),
                             T_DJV, T_RDJV, t - 1, j - 1);
            if (j == nj)
                dfdynnf = (b.bc[3] != LES_BCT_INTERFACE_D)
                              ? dfdynf
                              : (R)GR[(long)(A.link[bi * 6 + 3]) * 6 * gst + 2 * gst + (i - 1) + (long)gm * (k - 1)];
            else
                dfdynnf = QD(SC(t + 2, j + 2) - sn, T_DJV, T_RDJV, t + 2, j + 2);
#undef QD
            const R rpij = TB(T_RP, t, j);
            const R rrpij = FAST ? TB(T_RRP, t, j) : zero;
#define QZ(x, dk_, rdk_) (FAST ? (x) * (rrpij * (rdk_)) : (x) / (rpij * (dk_)))
            const R dfdzlf = QZ(s0 - sl, dkp_m2, rdkp_m2);
            const R dfdzrf = QZ(sr - s0, dkp_m1, rdkp_m1);
            if (k == 2)
                dfdzllf = (b.bc[4] != LES_BCT_INTERFACE_D)
                              ? dfdzlf
                              : (R)GR[(long)(A.link[bi * 6 + 4]) * 6 * gst + 5 * gst + (i - 1) + (long)gm * (j - 1)];
            else
                dfdzllf = QZ(sl - (R)fresh<S>(m2, A.scnew + e3(k - 2, t, j), A.err, limit), dkp_m3, rdkp_m3);
            if (k == nk)
                dfdzrrf = (b.bc[5] != LES_BCT_INTERFACE_D)
                              ? dfdzrf
                              : (R)GR[(long)(A.link[bi * 6 + 5]) * 6 * gst + 4 * gst + (i - 1) + (long)gm * (j - 1)];
            else
                dfdzrrf = QZ(at(GR_P2, 0, t, j) - sr, dkp_0, rdkp_0);
#undef QZ
            // the limiters' slope ratios: an FP32 build divides with
            // __fdividef (2 ulp; the ratio only enters min(4 r, 1)), the
            // FP64 builds as the reference does
            auto ratio = [](R a, R b) -> R {
                if constexpr (sizeof(R) == 4 && FAST) return __fdividef(a, b);
                else return a / b;
            };
            const R rwst = (uwf >= zero) ? ratio(dfdxwwf + small, dfdxwf + small) : ratio(dfdxef + small, dfdxwf + small);
            const R rest = (uef > zero) ? ratio(dfdxwf + small, dfdxef + small) : ratio(dfdxeef + small, dfdxef + small);
            const R rsth = (vsf >= zero) ? ratio(dfdyssf + small, dfdysf + small) : ratio(dfdynf + small, dfdysf + small);
            const R rnth = (vnf > zero) ? ratio(dfdysf + small, dfdynf + small) : ratio(dfdynnf + small, dfdynf + small);
            const R rlft = (wlf >= zero) ? ratio(dfdzllf + small, dfdzlf + small) : ratio(dfdzrf + small, dfdzlf + small);
            const R rrht = (wrf > zero) ? ratio(dfdzlf + small, dfdzrf + small) : ratio(dfdzrrf + small, dfdzrf + small);
            const R limw = fmax(zero, fmin(lambda * rwst, one));
            const R lime = fmax(zero, fmin(lambda * rest, one));
            const R lims = fmax(zero, fmin(lambda * rsth, one));
            const R limn = fmax(zero, fmin(lambda * rnth, one));
            const R liml = fmax(zero, fmin(lambda * rlft, one));
            const R limr = fmax(zero, fmin(lambda * rrht, one));
            R fwf, fef, fsf, fnf, flf, frf;
            if (uwf > zero) fwf = sw + half * limw * (s0 - sw);
            else if (uwf < zero) fwf = s0 + half * limw * (sw - s0);
            else fwf = half * (s0 + sw);
            if (uef > zero) fef = s0 + half * lime * (se - s0);
            else if (uef < zero) fef = se + half * lime * (s0 - se);
            else fef = half * (s0 + se);
            if (vsf > zero) fsf = ss + half * lims * (s0 - ss);
            else if (vsf < zero) fsf = s0 + half * lims * (ss - s0);
            else fsf = half * (s0 + ss);
            if (vnf > zero) fnf = s0 + half * limn * (sn - s0);
            else if (vnf < zero) fnf = sn + half * limn * (s0 - sn);
            else fnf = half * (s0 + sn);
            if (wlf > zero) flf = sl + half * liml * (s0 - sl);
            else if (wlf < zero) flf = s0 + half * liml * (sl - s0);
            else flf = half * (s0 + sl);
            if (wrf > zero) frf = s0 + half * limr * (sr - s0);
            else if (wrf < zero) frf = sr + half * limr * (s0 - sr);
            else frf = half * (s0 + sr);
            const R areawf = TB(T_RDJU, t, j) * dkw_k;
            const R areaef = TB(T_RDJU, t + 1, j) * dkw_k;
            const R areasf = TB(T_RDIV, t, j) * dkw_k;
            const R areanf = TB(T_RDIV, t + 1, j + 1) * dkw_k;
            const R areak = TB(T_DIDJP, t, j);
            const R vol = TB(T_RDIDJP, t, j) * dkw_k;
            const R gwf = rhowf * uwf * fwf * areawf;
            const R gef = rhoef * uef * fef * areaef;
            const R gsf = rhosf * vsf * fsf * areasf;
            const R gnf = rhonf * vnf * fnf * areanf;
            const R glf = rholf * wlf * flf * areak;
            const R grf = rhorf * wrf * frf * areak;
            const R convf = -(gef - gwf) - (gnf - gsf) - (grf - glf);
            const R twf = gamwf * areawf * dfdxwf;
            const R tef = gamef * areaef * dfdxef;
            const R tsf = gamsf * areasf * dfdysf;
            const R tnf = gamnf * areanf * dfdynf;
            const R tlf = gamlf * areak * dfdzlf;
            const R trf = gamrf * areak * dfdzrf;
            const R difff = (tef - twf) + (tnf - tsf) + (trf - tlf);
            const R h = convf + difff;
            R tmp = s0 + dtime / (vol * rhop) * ((R)1.5 * h - half * at(GR_OWN, 1, t, j));
            if (tmp < zero) tmp = zero;
            if (tmp > one) tmp = one;
            // the new value: in the ring slot of plane t (read by later
            // planes of this tile) and in the new-value array (read by the
            // layers above and the tile above); the history in place
            slot(GR_OWN, 0, t, j) = (S)tmp;
            const long e = e3(k, t, j);
            st_strong(A.scnew + e, (S)tmp);
            A.f3[1][e] = (S)h;
        }
        // the copies still in flight (issued, never waited for) land before
        // the ring is reused or the CTA exits
        const long uend = ubase + (t - ts);  // groups issued: ubase .. uend-1
        if (producer && lane == 0)
            for (long w = max(ubase, uend - D); w < uend; w++) mbar_drain(&mbar[w % G], (unsigned)((w / G) & 1), A.err, limit);
        __syncthreads();
        ubase = uend;
        if (!ok) return;
    }
#undef SC
#undef TB
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

template <typename S>
void launch_init_new_t(const SkewBlk *sb, int nb, const S *old, S *nw, cudaStream_t st)
{
    k_init_new<S><<<dim3(2048, nb), 256, 0, st>>>(sb, old, nw);
    les::count_launch(1);
}

// dynamic shared memory of the ring for row width sw
template <typename R, typename S, bool FAST, int D>
int tiles_smem(int sw)
{
    return gbase(GR_N, FAST, D, sw, (int)sizeof(S)) * (int)sizeof(S);
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
void launch_sweep_init_new(const SkewBlk *sb, int nb, const double *old, double *nw, cudaStream_t st)
{
    launch_init_new_t<ST>(sb, nb, old, nw, st);
}
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
void launch_sweep_init_new(const SkewBlk *sb, int nb, const float *old, float *nw, cudaStream_t st)
{
    les_fast::launch_init_new_t<float>(sb, nb, old, nw, st);
}
int sweep_tiles_smem(int sw) { return les_fast::tiles_smem<float, float, true, kSweepDepth>(sw); }
int sweep_tiles_max_ctas(int sw, int nthr) { return les_fast::tiles_max_ctas<float, float, true, kSweepDepth>(sw, nthr); }
cudaError_t launch_sweep_tiles(const SweepArgs<float> &a, double dtime, long limit, int nctas, int nthr,
                               cudaStream_t st)
{
    return les_fast::launch_tiles_t<float, float, true, kSweepDepth>(a, dtime, limit, nctas, nthr, st);
}
} // namespace les_f32
#endif
