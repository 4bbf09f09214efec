// k_metric.cu -- staggered-grid metrics on the device, FP64, -fmad=false.
//
// comp_metric (code/comp_metric.F:5-255): metric_block
// (code/metric_block2.F:9-280) for every block of a level, then the metric
// exchange on periodic/interface sides (code/metric_swap1.F,
// code/metric_swap2.F): pack every side, then unpack.  One thread per (i, j)
// point; the curvature terms need neighbouring lengths, so they run in a
// second kernel after the first has finished.
#include "k_common.cuh"
#include "kernels.h"

enum { M_DIP, M_DIU, M_DIV, M_DIX, M_RDIP, M_RDIV, M_RDIX, M_DJP, M_DJU, M_DJV, M_DJX, M_RDJP,
       M_RDJU, M_RDJX, M_HIJP, M_HJIP, M_HKIP, M_HKJP, M_HIJU, M_HJIU, M_HKIU, M_HKJU, M_HIJV,
       M_HJIV, M_HKIV, M_HKJV, M_RP, M_RU, M_RV, M_DIDJP, M_RDIDJP, M_DIDJU, M_RDIDJU, M_DJDIV,
       M_RDJDIV };

struct MetricPtrs {
    double *m[35];
};

// metric_swap1/2 move these 34 arrays (rdidjp is not exchanged)
__constant__ int c_swapped[34] = {M_DIP, M_DIU, M_DIV, M_DIX, M_RDIP, M_RDIV, M_RDIX, M_DJP, M_DJU,
                                  M_DJV, M_DJX, M_RDJP, M_RDJU, M_RDJX, M_HIJP, M_HJIP, M_HKIP,
                                  M_HKJP, M_HIJU, M_HJIU, M_HKIU, M_HKJU, M_HIJV, M_HJIV, M_HKIV,
                                  M_HKJV, M_RP, M_RU, M_RV, M_DIDJP, M_DIDJU, M_RDIDJU, M_DJDIV,
                                  M_RDJDIV};

struct MetBlk {
    int n[3];
    long off2, off1k, offxy, offz;
};

// metric_block2.F:67-241 for one (i, j); all 35 arrays are written (the
// curvature terms get their zero here and their value in k_metric_h)
__global__ void k_metric_main(const MetBlk *__restrict__ mb, const double *__restrict__ x,
                              const double *__restrict__ y, MetricPtrs P, double rad_on)
{
    const MetBlk b = mb[blockIdx.y];
    int nip1 = b.n[0], njp1 = b.n[1], nip2 = nip1 + 1;
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)nip1 * njp1) return;
    int i = (int)(q % nip1) + 1, j = (int)(q / nip1) + 1;
    double rad_off = 1. - rad_on;
    const double *X = x + b.offxy, *Y = y + b.offxy;
#define XV(ii, jj) X[((ii) - 1) + (long)nip2 * ((jj) - 1)]
#define YV(ii, jj) Y[((ii) - 1) + (long)nip2 * ((jj) - 1)]
    int ip1 = min(i + 1, nip1), im1 = max(i - 1, 1), jp1 = min(j + 1, njp1), jm1 = max(j - 1, 1);
    double x_ij = XV(i, j), x_ip1j = XV(ip1, j), x_ijp1 = XV(i, jp1), x_ip1jp1 = XV(ip1, jp1);
    double x_im1j = XV(im1, j), x_im1jp1 = XV(im1, jp1), x_ijm1 = XV(i, jm1), x_ip1jm1 = XV(ip1, jm1);
    double y_ij = YV(i, j), y_ip1j = YV(ip1, j), y_ijp1 = YV(i, jp1), y_ip1jp1 = YV(ip1, jp1);
    double y_im1j = YV(im1, j), y_im1jp1 = YV(im1, jp1), y_ijm1 = YV(i, jm1), y_ip1jm1 = YV(ip1, jm1);
#undef XV
#undef YV
    double xu_ij = 0.5 * (x_ij + x_ijp1), yu_ij = 0.5 * (y_ij + y_ijp1);
    double xu_ijm1 = 0.5 * (x_ij + x_ijm1), yu_ijm1 = 0.5 * (y_ij + y_ijm1);
    double xu_ip1j = 0.5 * (x_ip1j + x_ip1jp1), yu_ip1j = 0.5 * (y_ip1j + y_ip1jp1);
    double xv_ij = 0.5 * (x_ij + x_ip1j), yv_ij = 0.5 * (y_ij + y_ip1j);
    double xv_im1j = 0.5 * (x_ij + x_im1j), yv_im1j = 0.5 * (y_ij + y_im1j);
    double xv_ijp1 = 0.5 * (x_ijp1 + x_ip1jp1), yv_ijp1 = 0.5 * (y_ijp1 + y_ip1jp1);
    double xp_ij = 0.25 * (x_ij + x_ip1j + x_ijp1 + x_ip1jp1);
    double yp_ij = 0.25 * (y_ij + y_ip1j + y_ijp1 + y_ip1jp1);
    double xp_ijm1 = 0.25 * (x_ij + x_ip1j + x_ijm1 + x_ip1jm1);
    double yp_ijm1 = 0.25 * (y_ij + y_ip1j + y_ijm1 + y_ip1jm1);
    double xp_im1j = 0.25 * (x_ij + x_im1j + x_ijp1 + x_im1jp1);
    double yp_im1j = 0.25 * (y_ij + y_im1j + y_ijp1 + y_im1jp1);
    double rp_ij = yp_ij * rad_on + rad_off;
    double ru_ij = yu_ij * rad_on + rad_off;
    double rv_ij = yv_ij * rad_on + rad_off;
    double rx_ij = y_ij * rad_on + rad_off;
    long p = b.off2 + q;
    double dip = sqrt((xu_ip1j - xu_ij) * (xu_ip1j - xu_ij) + (yu_ip1j - yu_ij) * (yu_ip1j - yu_ij));
    double diu = sqrt((xp_ij - xp_im1j) * (xp_ij - xp_im1j) + (yp_ij - yp_im1j) * (yp_ij - yp_im1j));
    double div = sqrt((x_ip1j - x_ij) * (x_ip1j - x_ij) + (y_ip1j - y_ij) * (y_ip1j - y_ij));
    double dix = sqrt((xv_ij - xv_im1j) * (xv_ij - xv_im1j) + (yv_ij - yv_im1j) * (yv_ij - yv_im1j));
    double djp = sqrt((xv_ijp1 - xv_ij) * (xv_ijp1 - xv_ij) + (yv_ijp1 - yv_ij) * (yv_ijp1 - yv_ij));
    double dju = sqrt((x_ijp1 - x_ij) * (x_ijp1 - x_ij) + (y_ijp1 - y_ij) * (y_ijp1 - y_ij));
    double djv = sqrt((xp_ij - xp_ijm1) * (xp_ij - xp_ijm1) + (yp_ij - yp_ijm1) * (yp_ij - yp_ijm1));
    double djx = sqrt((xu_ij - xu_ijm1) * (xu_ij - xu_ijm1) + (yu_ij - yu_ijm1) * (yu_ij - yu_ijm1));
    P.m[M_RU][p] = ru_ij;
    P.m[M_RV][p] = rv_ij;
    P.m[M_RP][p] = rp_ij;
    P.m[M_DIP][p] = dip;
    P.m[M_DIU][p] = diu;
    P.m[M_DIV][p] = div;
    P.m[M_DIX][p] = dix;
    P.m[M_RDIP][p] = rp_ij * dip;
    P.m[M_RDIV][p] = rv_ij * div;
    P.m[M_RDIX][p] = rx_ij * dix;
    P.m[M_DJP][p] = djp;
    P.m[M_DJU][p] = dju;
    P.m[M_DJV][p] = djv;
    P.m[M_DJX][p] = djx;
    P.m[M_RDJP][p] = rp_ij * djp;
    P.m[M_RDJU][p] = ru_ij * dju;
    P.m[M_RDJX][p] = rx_ij * djx;
    double didjp = dip * djp;
    P.m[M_DIDJP][p] = didjp;
    P.m[M_DIDJU][p] = diu * dju;
    P.m[M_DJDIV][p] = djv * div;
    P.m[M_RDIDJP][p] = rp_ij * didjp;
    P.m[M_RDIDJU][p] = diu * (ru_ij * dju);
    P.m[M_RDJDIV][p] = djv * (rv_ij * div);
    for (int h = M_HIJP; h <= M_HKJV; h++) P.m[h][p] = 0.;
}

// metric_block2.F:247-253 and 258-277.  hkju and hkiv use the corner
// (nip1, njp1) coordinates left over from the first loop, whose difference
// is exactly zero, so both are 0 * rad_on / (... + tiny).
__global__ void k_metric_h(const MetBlk *__restrict__ mb, const double *__restrict__ z,
                           double *__restrict__ dkp, double *__restrict__ dkw, MetricPtrs P,
                           double rad_on)
{
    const MetBlk b = mb[blockIdx.y];
    int nip1 = b.n[0], njp1 = b.n[1], nkp1 = b.n[2];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const double tiny = 1.0e-30;
    if (q < nkp1) {
        int k = (int)q + 1;
        int kp1 = min(k + 1, nkp1), km1 = max(k - 1, 1);
        const double *t = z + b.offz;
        dkp[b.off1k + k - 1] = t[kp1 - 1] - t[k - 1];
        dkw[b.off1k + k - 1] = (t[kp1 - 1] - t[km1 - 1]) * 0.5;
    }
    if (q >= (long)nip1 * njp1) return;
    int i = (int)(q % nip1) + 1, j = (int)(q / nip1) + 1;
    if (i < 2 || i > nip1 - 1 || j < 2 || j > njp1 - 1) return;
    long p = b.off2 + q;
    long jo = nip1;
    double *const *m = P.m;
    m[M_HIJP][p] = (m[M_DIV][p + jo] - m[M_DIV][p]) / (m[M_DIDJP][p] + tiny);
    m[M_HJIP][p] = (m[M_DJU][p + 1] - m[M_DJU][p]) / (m[M_DIDJP][p] + tiny);
    m[M_HKIP][p] = (m[M_RU][p + 1] - m[M_RU][p]) / (m[M_RDIP][p] + tiny);
    m[M_HKJP][p] = (m[M_RV][p + jo] - m[M_RV][p]) / (m[M_RDJP][p] + tiny);
    m[M_HIJU][p] = (m[M_DIX][p + jo] - m[M_DIX][p]) / (m[M_DIDJU][p] + tiny);
    m[M_HJIU][p] = (m[M_DJP][p] - m[M_DJP][p - 1]) / (m[M_DIDJU][p] + tiny);
    m[M_HKIU][p] = (m[M_RP][p] - m[M_RP][p - 1]) / (m[M_RU][p] * m[M_DIU][p] + tiny);
    m[M_HKJU][p] = 0.0 * rad_on / (m[M_RDJU][p] + tiny);
    m[M_HIJV][p] = (m[M_DIP][p] - m[M_DIP][p - jo]) / (m[M_DJDIV][p] + tiny);
    m[M_HJIV][p] = (m[M_DJX][p + 1] - m[M_DJX][p]) / (m[M_DJDIV][p] + tiny);
    m[M_HKIV][p] = 0.0 * rad_on / (m[M_RDIV][p] + tiny);
    m[M_HKJV][p] = (m[M_RP][p] - m[M_RP][p - jo]) / (m[M_RV][p] * m[M_DJV][p] + tiny);
}

// One side of one block in the metric exchange.  For i sides the line is a
// column (io = 1, jo = nip1, length njp1), for j sides a row.
struct MetFace {
    long src2, dst2;   // 0-based first element of the packed / ghost line
    long stride;       // step along the own (ghost) line
    long sstride;      // step along the partner's (packed) line
    int len;           // line length
    long srck, dstk;   // 1-D (dkp, dkw) element for k sides, -1 otherwise
};

__global__ void k_metric_swap(const MetFace *__restrict__ fc, int nf, MetricPtrs P,
                              double *__restrict__ dkp, double *__restrict__ dkw,
                              double *__restrict__ buf, long slot, int phase)
{
    const MetFace f = fc[blockIdx.y];
    double *b = buf + slot * blockIdx.y;
    if (f.srck >= 0) {
        if (threadIdx.x == 0 && blockIdx.x == 0) {
            if (phase == 0) { b[0] = dkp[f.srck]; b[1] = dkw[f.srck]; }
            else { dkp[f.dstk] = b[0]; dkw[f.dstk] = b[1]; }
        }
        return;
    }
    long n = (long)f.len * 34;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        int a = (int)(q % 34);
        long jj = q / 34;
        int arr = c_swapped[a];
        if (phase == 0) b[q] = P.m[arr][f.src2 + f.sstride * jj];
        else P.m[arr][f.dst2 + f.stride * jj] = b[q];
    }
}

namespace les {

void launch_metric(const void *metblk, int nb, long maxij, long maxk, const double *x,
                   const double *y, const double *z, double *const *m, double *dkp, double *dkw,
                   int gotrad, cudaStream_t st)
{
    MetricPtrs P;
    for (int a = 0; a < 35; a++) P.m[a] = m[a];
    double rad_on = gotrad ? 1. : 0.;
    long n = maxij > maxk ? maxij : maxk;
    unsigned gx = (unsigned)((n + 127) / 128);
    k_metric_main<<<dim3(gx, nb), 128, 0, st>>>((const MetBlk *)metblk, x, y, P, rad_on);
    k_metric_h<<<dim3(gx, nb), 128, 0, st>>>((const MetBlk *)metblk, z, dkp, dkw, P, rad_on);
    count_launch(2);
}

void launch_metric_swap(const void *faces, int nf, long maxlen, double *const *m, double *dkp,
                        double *dkw, double *buf, long slot, int phase, cudaStream_t st)
{
    if (nf == 0) return;
    MetricPtrs P;
    for (int a = 0; a < 35; a++) P.m[a] = m[a];
    unsigned gx = (unsigned)((maxlen * 34 + 255) / 256);
    if (gx > 64) gx = 64;
    if (gx < 1) gx = 1;
    k_metric_swap<<<dim3(gx, nf), 256, 0, st>>>((const MetFace *)faces, nf, P, dkp, dkw, buf, slot, phase);
    count_launch(1);
}

size_t metblk_size() { return sizeof(MetBlk); }
size_t metface_size() { return sizeof(MetFace); }

void fill_metblk(void *dst, int idx, const int *n, long off2, long off1k, long offxy, long offz)
{
    MetBlk *b = (MetBlk *)dst + idx;
    for (int d = 0; d < 3; d++) b->n[d] = n[d];
    b->off2 = off2;
    b->off1k = off1k;
    b->offxy = offxy;
    b->offz = offz;
}

void fill_metface(void *dst, int idx, long src2, long dst2, long stride, long sstride, int len,
                  long srck, long dstk)
{
    MetFace *f = (MetFace *)dst + idx;
    f->src2 = src2;
    f->dst2 = dst2;
    f->stride = stride;
    f->sstride = sstride;
    f->len = len;
    f->srck = srck;
    f->dstk = dstk;
}

} // namespace les
