// lester_noalloc.cu -- lester_norms_noalloc: the residual and norms of one
// block of the pressure system with no device allocation at all.
//
// Who needs it: a host that must not allocate device memory at the point
// of the call -- code running inside a CUDA stream capture (cudaMalloc and
// cudaFree are not permitted there), a real-time loop with a fixed memory
// budget, or a host that owns all device memory through its own pool and
// forbids allocations by libraries.  lester_norms needs lester_gpu_init,
// which allocates the library's tables and its reduction scratch; this
// variant needs neither.
//
// Its scratch is a file-scope static device array of fixed size: one slot
// of 4 partial sums per 256-point CTA plus 8 result slots.  The largest
// block it accepts therefore has LES_NOALLOC_MAX_POINTS interior points;
// larger blocks are rejected with LES_ERR_SIZE before any device work.
// Every call writes every scratch slot that it later reads, so nothing in
// the scratch has to start at zero.  The scratch is shared by all calls on
// a device: calls whose work overlaps on the GPU (two streams, or two host
// threads) race on it and must be serialised by the caller.
//
// The device address of the scratch is looked up once per device with
// cudaGetSymbolAddress, with that device current, on the first call made
// while it is current.  That first call should come before any stream
// capture is begun.
//
// The arithmetic is that of k_norms / k_norms_final (FP64, no FMA
// contraction, same reduction order), so the results equal lester_norms on
// the same single-block input.
#include <mutex>

#include "k_common.cuh"
#include "lester_ctx.h"

namespace {

constexpr int kThreads = 256;
constexpr long kMaxParts = LES_NOALLOC_MAX_POINTS / kThreads;

static __device__ __align__(256) double g_noalloc_scratch[4 * kMaxParts + 8];

__global__ void __launch_bounds__(kThreads)
    k_norms_noalloc(BlkDev b, const double *__restrict__ ap, const double *__restrict__ aw,
                    const double *__restrict__ ae, const double *__restrict__ as,
                    const double *__restrict__ an, const double *__restrict__ al,
                    const double *__restrict__ ar, const double *__restrict__ x,
                    const double *__restrict__ bb, double *__restrict__ residu,
                    double *__restrict__ partial)
{
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    double v[4] = {0., 0., 0., 0.};
    if (q < b.ncell) {
        int i, j, k;
        long p = decode_interior(b, q, i, j, k);
        long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
        double var = x[p];
        double res = bb[p] - ap[p] * var + aw[p] * x[p - 1] + ae[p] * x[p + 1] +
                     as[p] * x[p - jo] + an[p] * x[p + jo] + al[p] * x[p - ko] +
                     ar[p] * x[p + ko];
        double err = res / ap[p];
        v[0] = res * res;
        v[1] = bb[p] * bb[p];
        v[2] = err * err;
        v[3] = var * var;
        residu[p] = res;
    }
    block_reduce_store<4>(v, partial + 4 * (long)blockIdx.x);
}

// out[0..4) = sqrt(sum / npts), out[4..8) = raw sums; a zero var norm
// becomes 1 (code/norms.F:398)
__global__ void k_norms_noalloc_final(const double *__restrict__ partial, long nparts,
                                      double rnpts, double *__restrict__ out)
{
    double v[4] = {0., 0., 0., 0.};
    for (long t = threadIdx.x; t < nparts; t += blockDim.x)
        for (int c = 0; c < 4; c++) v[c] += partial[t * 4 + c];
    __shared__ double res[4];
    block_reduce_store<4>(v, res);
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int c = 0; c < 4; c++) {
            out[4 + c] = res[c];
            out[c] = sqrt(res[c] * rnpts);
        }
        if (out[3] == 0.) out[3] = 1.;
    }
}

constexpr int kMaxDev = 64;
std::mutex g_setup_mu;
double *g_scratch_dev[kMaxDev] = {};

// device address of the scratch on the current device (first call per
// device looks it up)
int scratch_address(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return les::set_err(LES_ERR_CUDA, "lester_norms_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    }
    if (dev < 0 || dev >= kMaxDev) return les::set_err(LES_ERR_ARG, "lester_norms_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_dev[dev]) {
        double *p = nullptr;
        e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return les::set_err(LES_ERR_CUDA, "lester_norms_noalloc: cudaGetSymbolAddress: %s",
                                cudaGetErrorString(e));
        }
        g_scratch_dev[dev] = p;
    }
    *out = g_scratch_dev[dev];
    return 0;
}

} // namespace

extern "C" int lester_norms_noalloc(const int *nijkp1, const double *ap, const double *aw,
                                    const double *ae, const double *as, const double *an,
                                    const double *al, const double *ar, const double *x,
                                    const double *b, double *residu, double *res_norm,
                                    double *rhs_norm, double *err_norm, double *var_norm,
                                    void *stream)
{
    using les::set_err;
    if (!nijkp1) return set_err(LES_ERR_ARG, "lester_norms_noalloc: nijkp1 is NULL");
    for (int d = 0; d < 3; d++)
        if (nijkp1[d] < 3) return set_err(LES_ERR_ARG, "lester_norms_noalloc: nijkp1[%d] = %d < 3", d, nijkp1[d]);
    long ncell = (long)(nijkp1[0] - 2) * (nijkp1[1] - 2) * (nijkp1[2] - 2);
    if (ncell > LES_NOALLOC_MAX_POINTS)
        return set_err(LES_ERR_SIZE,
                       "lester_norms_noalloc: %ld interior points exceed the fixed scratch limit of %ld "
                       "(use lester_norms for larger blocks)",
                       ncell, (long)LES_NOALLOC_MAX_POINTS);
    const double *ptr[] = {ap, aw, ae, as, an, al, ar, x, b, residu};
    for (const double *p : ptr)
        if (!p) return set_err(LES_ERR_ARG, "lester_norms_noalloc: NULL array");
    if (!res_norm || !rhs_norm || !err_norm || !var_norm)
        return set_err(LES_ERR_ARG, "lester_norms_noalloc: NULL norm output");
    for (const double *p : ptr) {
        cudaPointerAttributes at;
        cudaError_t e = cudaPointerGetAttributes(&at, p);
        if (e != cudaSuccess || (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
            cudaGetLastError();
            return set_err(LES_ERR_ARG, "lester_norms_noalloc: arrays must be device memory");
        }
    }
    double *scratch = nullptr;
    int r = scratch_address(&scratch);
    if (r) return r;
    cudaStream_t st = (cudaStream_t)stream;
    BlkDev blk{};
    for (int d = 0; d < 3; d++) blk.n[d] = nijkp1[d];
    blk.ncell = ncell;
    unsigned gx = (unsigned)((ncell + kThreads - 1) / kThreads);
    double *out = scratch + 4 * kMaxParts;
    k_norms_noalloc<<<gx, kThreads, 0, st>>>(blk, ap, aw, ae, as, an, al, ar, x, b, residu, scratch);
    k_norms_noalloc_final<<<1, kThreads, 0, st>>>(scratch, (long)gx, 1.0 / (double)ncell, out);
    double h[8];
    cudaError_t e = cudaMemcpyAsync(h, out, sizeof h, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(LES_ERR_CUDA, "lester_norms_noalloc: %s", cudaGetErrorString(e));
    }
    *res_norm = h[0];
    *rhs_norm = h[1];
    *err_norm = h[2];
    *var_norm = h[3];
    return 0;
}
