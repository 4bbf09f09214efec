// k_virtbc.cu -- wall ghost velocities and van Driest damping (FP64,
// -fmad=false): set_virt_bc (code/set_virt_bc.F:55-273) and the velocity
// branches of set_virt_bc_block (code/set_virt_bc_block.F:69-435).
//
// One launch per wall side, sides in the reference's order, so that where
// two sides share an edge the later one wins as in the sequential loops.
// Within a side every point of the ghost plane (or, for the u south/north
// damping, of the half-domain damping planes) is independent.
// At i = 1 of the u south/north branch the reference averages rho with the
// element before the slice; rho(i) is used there (corner ghost only).
#include "k_common.cuh"
#include "kernels.h"

__device__ __forceinline__ double sign1(double b) { return b >= 0.0 ? 1.0 : -1.0; }

// u, south/north wall: damping over half the block from the wall, ghost
// value on the first plane (set_virt_bc_block.F:81-168)
__global__ void k_vbc_u_sn(const BlkDev *__restrict__ blk, int side, unsigned long long wallmask,
                           VbcArgs A, double visc, double kappa, double aplus, double ylam,
                           double value)
{
    const BlkDev b = blk[blockIdx.y];
    if (!((wallmask >> blockIdx.y) & 1ull)) return;
    int n0 = b.n[0], n1 = b.n[1], n2 = b.n[2];
    int half = n1 / 2 + 1;  // kvd = kstart .. kstart +- n1/2
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)n0 * n2 * half) return;
    int i = (int)(q % n0) + 1;
    long t = q / n0;
    int k = (int)(t % n2) + 1;
    int m = (int)(t / n2);
    int k1 = (side == 3) ? 2 : n1;
    int step = (side == 3) ? 1 : -1;
    int kvd = k1 + step * m;
    int kref = (side == 3) ? kvd - 1 : kvd;
    long jo = n0, ko = (long)n0 * n1;
    long ijk = b.off3 + (i - 1) + jo * (kref - 1) + ko * (k - 1);
    long nx = ijk + (side == 3 ? jo : -jo);
    const double *R = A.rho;
    double rw = (i > 1) ? R[ijk - 1] : R[ijk];
    double rwn = (i > 1) ? R[nx - 1] : R[nx];
    double rhof = 0.25 * (R[ijk] + R[nx] + rw + rwn);
    double twv = A.tw[A.off_ki[blockIdx.y] + (k - 1) + (long)n2 * (i - 1)];
    double tw_mean = fabs(twv);
    double ut = sqrt(tw_mean / rhof);
    long o2 = b.off2;
    double dist = 0.5 * A.dju[o2 + (i - 1) + (long)n0 * (k1 - 1)];
    if (m > 0)
        for (int kk = k1 + step; step > 0 ? kk <= kvd : kk >= kvd; kk += step)
            dist = dist + A.djx[o2 + (i - 1) + (long)n0 * (kk - 1)];
    double yp = dist * ut * rhof / visc;
    double d = 1. - exp(-yp / aplus);
    A.vdd[nx] = d < 1.0 ? d : 1.0;
    if (m == 0) {
        double snwall = (side == 4) ? -1. : 1.;
        if (yp > ylam)
            A.f[ijk] = A.f[nx] - snwall * sign1(twv) * ut * A.djx[o2 + (i - 1) + (long)n0 * (k1 - 1)] / (kappa * dist);
        else
            A.f[ijk] = 2. * value - A.f[nx];
    }
}

// every other velocity/side combination: one ghost plane
// (set_virt_bc_block.F:172-430)
__global__ void k_vbc_plane(const BlkDev *__restrict__ blk, int iva, int side,
                            unsigned long long wallmask, unsigned long long initmask, VbcArgs A,
                            double visc, double kappa, double aplus, double ylam, double value)
{
    const BlkDev b = blk[blockIdx.y];
    if (!((wallmask >> blockIdx.y) & 1ull)) return;
    const int cyc1[2][4] = {{0, 2, 1, 1}, {0, 3, 3, 2}};
    long st[4] = {0, 1, b.n[0], (long)b.n[0] * b.n[1]};
    int nn[4] = {0, b.n[0], b.n[1], b.n[2]};
    int d3 = (side + 1) / 2, d1 = cyc1[0][d3], d2 = cyc1[1][d3];
    long io = st[d1], jo = st[d2], ko = st[d3];
    int nip1 = nn[d1], njp1 = nn[d2], nkp1 = nn[d3];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)nip1 * njp1) return;
    int i = (int)(q % nip1) + 1, j = (int)(q / nip1) + 1;
    int k, k1;
    long kko;
    if (side % 2 == 1) { k = 1; k1 = 2; kko = ko; }
    else { k = nkp1; k1 = nkp1; kko = -ko; }
    long koff = 1 + ko * (k - 1);
    long base = b.off3 - 1;  // 1-based block index -> field position
    long ijk = base + io * (i - 1) + jo * (j - 1) + koff, nx = ijk + kko;
    const double *R = A.rho;
    // the running "last" densities of the source loops
    bool i_outer = (iva == 2 && side >= 5) || iva == 3;
    double rl, rln;
    if (i_outer) {
        if (j == 1) { rl = R[base + koff]; rln = R[base + koff + kko]; }
        else { rl = R[ijk - jo]; rln = R[nx - jo]; }
    } else {
        if (i == 1) { rl = R[ijk]; rln = R[nx]; }
        else { rl = R[ijk - io]; rln = R[nx - io]; }
    }
    double rhof = 0.25 * (R[ijk] + R[nx] + rl + rln);
    long o2 = b.off2, o1 = b.off1k;
    int n0 = b.n[0];
    double dist, twv, wsgn, m1, m2 = 1.0;
    double wewall = (side == 2) ? -1. : 1., snwall = (side == 4) ? -1. : 1., lrwall = (side == 6) ? -1. : 1.;
    if (iva == 1) {  // L/R: (i, j) real
        long ij = o2 + (i - 1) + (long)n0 * (j - 1);
        dist = 0.5 * A.ru[ij] * A.dkp[o1 + k1 - 1];
        twv = A.tw[o2 + (i - 1) + (long)n0 * (j - 1)];  // (i, j) wall array, level-1 offset
        wsgn = lrwall;
        m1 = A.ru[ij];
        m2 = A.dkw[o1 + k1 - 1];
    } else if (iva == 2 && side <= 2) {  // i over real j, j over real k
        long qq = o2 + (k1 - 1) + (long)nkp1 * (i - 1);
        dist = 0.5 * A.div_[qq];
        twv = A.tw[A.off_jk[blockIdx.y] + (j - 1) + (long)njp1 * (i - 1)];
        wsgn = wewall;
        m1 = A.dix[qq];
    } else if (iva == 2) {  // L/R
        long ij = o2 + (i - 1) + (long)n0 * (j - 1);
        dist = 0.5 * A.rv[ij] * A.dkp[o1 + k1 - 1];
        twv = A.tw[o2 + (i - 1) + (long)n0 * (j - 1)];  // (i, j) wall array, level-1 offset
        wsgn = lrwall;
        m1 = A.rv[ij];
        m2 = A.dkw[o1 + k1 - 1];
    } else if (side <= 2) {  // w, W/E
        long qq = o2 + (k1 - 1) + (long)nkp1 * (i - 1);
        dist = 0.5 * A.dip[qq];
        twv = A.tw[A.off_jk[blockIdx.y] + (j - 1) + (long)njp1 * (i - 1)];
        wsgn = wewall;
        m1 = A.diu[qq];
    } else {  // w, S/N: i real i, j real k
        long qq = o2 + (i - 1) + (long)nip1 * (k1 - 1);
        dist = 0.5 * A.djp[qq];
        twv = A.tw[A.off_ki[blockIdx.y] + (j - 1) + (long)njp1 * (i - 1)];
        wsgn = snwall;
        m1 = A.djv[qq];
    }
    double tw_mean = fabs(twv);
    double ut = sqrt(tw_mean / rhof);
    double yp = dist * ut * rhof / visc;
    double d = 1. - exp(-yp / aplus);
    double cur = ((initmask >> blockIdx.y) & 1ull) ? 0.0 : A.vdd[nx];
    A.vdd[nx] = d > cur ? d : cur;
    if (yp > ylam)
        A.f[ijk] = A.f[nx] - wsgn * sign1(twv) * ut * m1 * m2 / (kappa * dist);
    else
        A.f[ijk] = 2. * value - A.f[nx];
}

namespace les {

void launch_vbc_side(const BlkDev *blk, int nb, int iva, int side, unsigned long long wallmask,
                     unsigned long long initmask, const VbcArgs &a, long maxpts, double visc,
                     double kappa, double aplus, double ylam, double value, cudaStream_t st)
{
    unsigned gx = (unsigned)((maxpts + 127) / 128);
    if (iva == 1 && (side == 3 || side == 4))
        k_vbc_u_sn<<<dim3(gx, nb), 128, 0, st>>>(blk, side, wallmask, a, visc, kappa, aplus, ylam, value);
    else
        k_vbc_plane<<<dim3(gx, nb), 128, 0, st>>>(blk, iva, side, wallmask, initmask, a, visc, kappa, aplus,
                                                 ylam, value);
    count_launch(1);
}

} // namespace les
