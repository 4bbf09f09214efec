// k_common.cuh -- device-side descriptors and helpers shared by the kernels.
//
// Layout in HBM is the reference arena's: one FP64 array per field, blocks
// back to back, each block in Fortran order (i fastest) including one ghost
// layer per side; multigrid fields hold every level, level after level
// (code/set_offset.F:166-234).  A kernel that works on every block of a
// level takes the level's BlkDev table and runs a 2-D grid:
// gridDim.y = block, gridDim.x covers that block's points.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// Programmatic dependent launch (sm_90 and later): a kernel launched with
// launch_pdl may start while the kernel before it on the stream drains; it
// computes what depends on no earlier kernel of the chain (indices,
// couplings set up long before), then pdl_wait() until the kernel before
// it has finished and its writes are visible, then pdl_trigger() lets the
// next one start.  Launched without the attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

#define LES_BCT_WALL_D 1
#define LES_BCT_ZERO_GRAD_D 2
#define LES_BCT_TRACTION_D 6
#define LES_BCT_PERIODIC_D 12
#define LES_BCT_INTERFACE_D 13

constexpr int kMaxBlk = 64;  // blocks per grid (code/dim.inc maxbl, LES_MAXBL)

struct BlkDev {
    int n[3];      // nip1, njp1, nkp1 (points incl. ghosts)
    int bc[6];     // W E S N L R
    int mult[3];   // coarsening factor to the next level (1 or 2)
    long off3;     // 0-based start of this block in a 3-D field at this level
    long off2;     // 0-based start in a 2-D (i,j) metric at this level
    long off1k;    // 0-based start in a 1-D k metric at this level
    long ncell;    // interior points (nip1-2)(njp1-2)(nkp1-2)
    int comp;      // connected component (blocks joined by periodic/interface links)
    int pad_;
};

// One convective-outflow or fixed-inflow side at level 1: its exit plane
// along axis d1 (conv_exitbc.F:141-143) and, per variable 1..3, the
// set_loop_bound ranges (1-based, inclusive; index 0 unused)
struct SideJob {
    int blk, side, d1, conv;  // 0-based block, side 1..6, axis 1..3, 1 = convective
    int n[3];
    int plane;
    long off3, off2, off1k;
    int bnd[4][6];
};

// per exit axis d1 = 1..3 (index 0 unused): the metric conv_exitbc passes
// as dip / rp / dkp to conv_exitbc1_block for the variable being updated
struct ExitMetrics {
    const double *dm[4], *rm[4], *km[4];
};

// recycling: the running means and rms (read and written) and the target
// mean and rms profiles of u, v, w, indexed by j (1-D device arrays)
struct RecycProf {
    const double *mean[3], *rms[3], *prof[3], *rprof[3];
};

// the 16 running span averages of statistics.F (2-D, level-1 metric
// layout): um vm wm pm rhom ruv rvw rwu ruu rvv rww rrh fm rff sc1varm T_m
struct StatOut {
    double *f[16];
};

// slots of the SAVEd outflow values (conv_exitbc.F:78): per-side totals
// (index side 1..6), inflow and outflow sums, mass change
enum { EX_TTL = 0, EX_ARHO = 7, EX_IN = 14, EX_OUT = 15, EX_MCHG = 16, EX_N = 17 };

// One periodic/interface face of swap_sc (code/swap_sc0.F:92-133 and
// 239-283).  Own pack plane = first interior plane of (block, side); own
// ghost plane receives the partner face's pack plane.  Positions are 0-based
// indices into the 3-D field, strides are the in-plane (j, k) strides.
struct FaceDev {
    long pk, gh, jo, ko;      // own pack plane, own ghost plane, strides
    long ppk, pjo, pko;       // partner pack plane and its strides
    int nj, nk;               // plane size (equal on both sides)
    long woff, pwoff;         // own and partner slot in the pack buffer
    int skip;                 // edge rows a later side of this block rewrites:
                              // 1 = j first, 2 = j last, 4 = k first, 8 = k last
};

// separable factors of the fast-solver coefficients (k_fast.cu): coupling
// E(i,j,k) = E2(i,j) Ez(k), likewise N and R; 2-D tables in the metric
// layout (b.off2), 1-D in the k layout (b.off1k).  E2 == nullptr: unused.
template <typename T> struct MfTab {
    T *E2 = nullptr, *N2 = nullptr, *R2 = nullptr, *Ez = nullptr, *Nz = nullptr, *Rz = nullptr;
};
// the same factorisation of the level-1 FP64 couplings as double-float pairs
using DfTab = MfTab<float2>;

// Push-style halo of the fast solvers: for side s of a block whose first
// interior plane feeds a ghost plane (periodic or interface link), the
// ghost cell mirroring a point of that plane with 0-based coordinates c[]
// is gh + jo * c[a2] + ko * c[a3].  A kernel that updates a point on such a
// plane writes the new value to its mirror as well, so no separate halo
// launch is needed; face interiors only, as the 7-point operator reads.
struct PushDev {
    long gh, jo, ko;
    int a2, a3, valid;
};

// The (block, plane) pairs a 3-D launch walks along gridDim.z: entry z is
// (0-based block, 1-based plane); n entries.  Built per level for its
// interior planes (2 .. n[2] - 1) and for the planes 1 .. n[2] - 1 a
// prolongation from it walks, so that blocks of different extents waste
// no planes and no CTA divides by a plane count.
struct ZMap {
    const int2 *map = nullptr;
    int n = 0;
};

// A level of at most kGeoBlk blocks as a kernel parameter (constant
// bank): per block its points with ghosts, its offsets in the 3-D, 2-D and
// 1-D arrays, and its six ghost mirrors -- a half sweep then loads no
// descriptor from memory, and a point on a mirrored face writes its ghost
// without a dependent load.  Offsets fit 32 bits (the multigrid arrays
// hold fewer than 2^31 points).
constexpr int kGeoBlk = 8;
struct LevGeo {
    int nb;
    int n[kGeoBlk][3];
    int off3[kGeoBlk], off2[kGeoBlk], off1k[kGeoBlk];
    PushDev push[kGeoBlk][6];
};

template <typename T>
__device__ __forceinline__ void push_ghosts(const PushDev *__restrict__ pd, const BlkDev &b, int i,
                                            int j, int k, T val, T *__restrict__ x)
{
    const int c[3] = {i - 1, j - 1, k - 1};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if (c[d] == 1) {
            const PushDev &P = pd[2 * d];
            if (P.valid) x[P.gh + P.jo * c[P.a2] + P.ko * c[P.a3]] = val;
        }
        if (c[d] == b.n[d] - 2) {
            const PushDev &P = pd[2 * d + 1];
            if (P.valid) x[P.gh + P.jo * c[P.a2] + P.ko * c[P.a3]] = val;
        }
    }
}

// The dense inverse of the V-cycle's bottom level (the fast solvers'
// coarse direct solve): n interior points in block-then-interior order,
// mt[h * n + g] = (A^-1)[g][h] (column-major, so that threads g read a
// column coalesced); n = 0 when the bottom level is smoothed instead.
constexpr int kDirectMax = 512;
template <typename T> struct CoarseDirect {
    const T *mt = nullptr;
    int n = 0;
};

// one multigrid level of the fast solvers, for kernels that walk levels
struct VLev {
    const BlkDev *blk;     // block table of the level (device)
    const PushDev *push;   // ghost mirrors, 6 per block
    const FaceDev *face;   // periodic / interface face copies
    int nface;
    int rb_push;           // red-black sweeps push (else copy the faces after each)
};

// true if in-plane element (j, k) (0-based) of face f is rewritten later by
// another side of the same block, so this face must leave it alone
__device__ __forceinline__ bool face_skips(const FaceDev &f, long j, long k)
{
    return ((f.skip & 1) && j == 0) || ((f.skip & 2) && j == f.nj - 1) ||
           ((f.skip & 4) && k == 0) || ((f.skip & 8) && k == f.nk - 1);
}

__device__ __forceinline__ bool is_per_or_int(int bc)
{
    return bc == LES_BCT_PERIODIC_D || bc == LES_BCT_INTERFACE_D;
}

// interior point number q -> (i, j, k) 1-based and 0-based field index
// (a block's interior count is below 2^31, checked at init, so the decode
// uses 32-bit divisions: a 64-bit division is a long emulated sequence)
__device__ __forceinline__ long decode_interior(const BlkDev &b, long q, int &i,
                                                int &j, int &k)
{
    const unsigned ni = (unsigned)(b.n[0] - 2), nj = (unsigned)(b.n[1] - 2), uq = (unsigned)q;
    const unsigned t = uq / ni;
    i = (int)(uq - t * ni) + 2;
    const unsigned t2 = t / nj;
    j = (int)(t - t2 * nj) + 2;
    k = (int)t2 + 2;
    return b.off3 + (i - 1) + (long)b.n[0] * ((j - 1) + (long)b.n[1] * (k - 1));
}

// Deterministic block reduction of NV doubles: warp shuffles in a fixed
// pattern, then warp 0 combines the per-warp sums in warp order.
template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double *out)
{
    __shared__ double sm[32][NV];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        v[q] = x;
    }
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; q++) sm[wid][q] = v[q];
    __syncthreads();
    if (wid == 0) {
        int nw = (blockDim.x + 31) >> 5;
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double x = lane < nw ? sm[lane][q] : 0.0;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) out[q] = x;
        }
    }
}

// ----------------------------------------------------- tiled scalar sweep
// (k_sweep.cu).  Skewed layout of a block: element (i, j, k) (1-based) of a
// 3-D field at sk3 + (k-1) layer + (i+j-2) vp + (j-1), of a 2-D table at
// sk2 + (i+j-2) vp + (j-1): plane t = i + j of a layer is one vector over j.
struct SkewBlk {
    int n[3];      // nip1, njp1, nkp1
    int vp;        // elements per plane vector: njp1 rounded up to 4
    int bc[6];
    long off3;     // FP64 3-D field offset of the block (level 1)
    long off2;     // FP64 2-D metric offset
    long off1k;    // 1-D k metric offset
    long sk3;      // skewed 3-D offset
    long sk2;      // skewed 2-D offset
    long layer;    // elements per skewed layer: (nip1 + njp1 - 1) vp
};

// one tile: block, layer k (2..nkp1-1), own rows j0..j1-1, and the tiles
// whose new values it reads: (block, k-1, same rows) and (block, k, rows
// below), -1 where there is none (they come before it in ticket order)
struct SweepTile {
    int blk, k, j0, j1, up_k, up_j;
};

constexpr int kSweepThreads = 256;  // rows per tile at most (one thread per row)
constexpr int kSweepDepth = 1;      // planes staged ahead

// sources (FP64, reference layout) and skewed destinations of one k_skew
// launch: up to 10 fields or tables
template <typename S> struct SkewPtrs {
    const double *src[10];
    S *dst[10];
};

template <typename S> struct SweepArgs {
    const SkewBlk *sb;
    const SweepTile *tiles;
    int ntile, sw;           // tiles; ring row width (elements)
    S *f3[8];                // skewed sc1 hsc1 u v w rho gamsc1 gamlam (old values; hsc1 updated)
    S *scnew;                // skewed new values of sc1 (field 8: interior -1 until computed, ghosts old)
    const S *f2[10];         // skewed diu djv rdju rdiv rp didjp rdidjp (+ 1/diu 1/djv 1/rp)
    const double *dkp, *dkw, *rdkp;
    const double *grad;      // interface gradients (set_gamsc1_bc planes)
    long gstride;
    int gm;
    const int *link;         // bl2bl, 0-based, 6 per block
    const void *tmaps;       // per block 4 TMA tensor maps (CUtensorMap, global memory): 3-D fields
                             // in boxes of 8, 4, 1 fields, the 2-D tables
    int *ticket;             // next tile to take
    int *err;                // a bounded wait gave up
};
