// lester_noalloc.cu -- lester_norms_noalloc: the residual and norms of one
// block of the pressure system with no device allocation at all.
//
// Who needs it: a host that must not allocate device memory when it calls
// this routine -- a solver embedded in a larger code that runs under a
// fixed device-memory budget, or one that owns all device memory through
// its own pool and forbids libraries to allocate behind its back, or a
// host that wants the norms of a block before (or without) setting up the
// library.  lester_norms needs lester_gpu_init, which allocates the
// library's tables and its reduction scratch; this variant needs neither.
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
// The call returns the four norms in host scalars: it queues its two
// kernels on `stream`, copies the 4 results back and waits for the stream.
//
// The device address of the scratch is looked up with cudaGetSymbolAddress,
// with the device current, on the first call in each CUDA context of a
// device (a cudaDeviceReset makes a new context, so the next call looks it
// up again).  That first call should come before any stream capture is
// begun.  Every array must be device memory of the current device.
//
// The arithmetic is that of k_norms / k_norms_final (FP64, no FMA
// contraction, same reduction order), so the results equal lester_norms on
// the same single-block input bit for bit.
#include <cuda.h>
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
// per device: the context the address was looked up in, and the address
struct ScratchSlot {
    unsigned long long ctx_id;
    double *ptr;
};
ScratchSlot g_scratch_dev[kMaxDev] = {};

typedef CUresult (*PfnCtxGetCurrent)(CUcontext *);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long *);
PfnCtxGetCurrent g_ctx_get_current = nullptr;
PfnCtxGetId g_ctx_get_id = nullptr;

// unique id of the current CUDA context (ids are never reused, so a
// context made by cudaDeviceReset has a new one); driver entry points are
// fetched through the runtime, so the library needs no libcuda link
int current_context_id(unsigned long long *id)
{
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
            cudaGetLastError();
            return les::set_err(LES_ERR_CUDA, "lester_norms_noalloc: driver context queries unavailable");
        }
        g_ctx_get_current = (PfnCtxGetCurrent)f1;
        g_ctx_get_id = (PfnCtxGetId)f2;
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx || g_ctx_get_id(ctx, id) != CUDA_SUCCESS)
        return les::set_err(LES_ERR_CUDA, "lester_norms_noalloc: no current CUDA context");
    return 0;
}

// device address of the scratch on the current device and context (the
// first call in each context looks it up)
int scratch_address(int dev, double **out)
{
    if (dev < 0 || dev >= kMaxDev) return les::set_err(LES_ERR_ARG, "lester_norms_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_setup_mu);
    unsigned long long id = 0;
    int r = current_context_id(&id);
    if (r) return r;
    ScratchSlot &s = g_scratch_dev[dev];
    if (!s.ptr || s.ctx_id != id) {
        double *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return les::set_err(LES_ERR_CUDA, "lester_norms_noalloc: cudaGetSymbolAddress: %s",
                                cudaGetErrorString(e));
        }
        s.ptr = p;
        s.ctx_id = id;
    }
    *out = s.ptr;
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
    int dev = 0;
    cudaError_t de = cudaGetDevice(&dev);
    if (de != cudaSuccess) {
        cudaGetLastError();
        return set_err(LES_ERR_CUDA, "lester_norms_noalloc: cudaGetDevice: %s", cudaGetErrorString(de));
    }
    for (const double *p : ptr) {
        cudaPointerAttributes at;
        cudaError_t e = cudaPointerGetAttributes(&at, p);
        if (e != cudaSuccess || (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
            cudaGetLastError();
            return set_err(LES_ERR_ARG, "lester_norms_noalloc: arrays must be device memory");
        }
        if (at.type == cudaMemoryTypeDevice && at.device != dev)
            return set_err(LES_ERR_ARG, "lester_norms_noalloc: an array lives on device %d, the current device is %d",
                           at.device, dev);
    }
    double *scratch = nullptr;
    int r = scratch_address(dev, &scratch);
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
