// k_exact.cu -- FP64 kernels of the pressure path that reproduce the
// reference's arithmetic operation for operation.
//
// This translation unit is compiled with -fmad=false: every product and sum
// is rounded separately, as in the reference's FP64 Fortran, and the
// operand order of each expression follows the cited source line, so
// results are bitwise equal to a non-contracting CPU evaluation.  Division
// and sqrt are IEEE round-to-nearest (nvcc defaults -prec-div/-prec-sqrt).
#include "k_common.cuh"
#include "kernels.h"

#define IDX3(b, i, j, k) ((b).off3 + ((i) - 1) + (long)(b).n[0] * (((j) - 1) + (long)(b).n[1] * ((k) - 1)))
#define IDX2(b, i, j) ((b).off2 + ((i) - 1) + (long)(b).n[0] * ((j) - 1))

// ------------------------------------------------------------------ swap_sc
// Two phases, exactly like code/swap_sc0.F: every face is packed before any
// ghost plane is written (edges and corners see the pre-exchange state).
// Where two ghost planes of one block share an edge, the reference writes
// it last from the higher-numbered side; the lower side skips it here so
// all faces can be unpacked in one launch with the same result.
__global__ void k_halo_pack(const FaceDev *__restrict__ fc, const double *__restrict__ var,
                            double *__restrict__ work)
{
    pdl_wait();
    pdl_trigger();
    const FaceDev f = fc[blockIdx.y];
    long n = (long)f.nj * f.nk;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        long k = q / f.nj, j = q - k * f.nj;
        work[f.woff + q] = var[f.pk + f.jo * j + f.ko * k];
    }
}

__global__ void k_halo_unpack(const FaceDev *__restrict__ fc, double *__restrict__ var,
                              const double *__restrict__ work)
{
    pdl_wait();
    pdl_trigger();
    const FaceDev f = fc[blockIdx.y];
    long n = (long)f.nj * f.nk;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        long k = q / f.nj, j = q - k * f.nj;
        if (face_skips(f, j, k)) continue;
        var[f.gh + f.jo * j + f.ko * k] = work[f.pwoff + q];
    }
}

// ------------------------------------------------------------------ coeff_p
// code/coeff_p_block.F:145-306 evaluated per interior point: aw/as/al are
// the neighbour's ae/an/ar (zero on the starting surfaces), ap is summed in
// the reference order, then the face corrections W,E,S,N,L,R in turn.
__global__ void k_coeff_p(const BlkDev *__restrict__ blk, const double *__restrict__ diu,
                          const double *__restrict__ djv, const double *__restrict__ rdiv,
                          const double *__restrict__ rdju, const double *__restrict__ didjp,
                          const double *__restrict__ rp, const double *__restrict__ dkp,
                          const double *__restrict__ dkw, double *__restrict__ ap,
                          double *__restrict__ aw, double *__restrict__ ae,
                          double *__restrict__ as, double *__restrict__ an,
                          double *__restrict__ al, double *__restrict__ ar)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long p = decode_interior(b, q, i, j, k);
    int ni = b.n[0] - 1, nj = b.n[1] - 1, nk = b.n[2] - 1;
    const double *dk = dkp + b.off1k, *dw = dkw + b.off1k;
    double cef = rdju[IDX2(b, i + 1, j)] / diu[IDX2(b, i + 1, j)];
    double cnf = rdiv[IDX2(b, i, j + 1)] / djv[IDX2(b, i, j + 1)];
    double crf = didjp[IDX2(b, i, j)] / rp[IDX2(b, i, j)];
    double vaw = 0.0, vas = 0.0, val = 0.0;
    if (i > 2) vaw = rdju[IDX2(b, i, j)] / diu[IDX2(b, i, j)] * dk[k - 1];
    if (j > 2) vas = rdiv[IDX2(b, i, j)] / djv[IDX2(b, i, j)] * dk[k - 1];
    if (k > 2) val = didjp[IDX2(b, i, j)] / rp[IDX2(b, i, j)] / dw[k - 1];
    double vae = cef * dk[k - 1];
    double van = cnf * dk[k - 1];
    double var_ = crf / dw[k];
    double vap = vaw + vae + vas + van + val + var_;
    if (i == 2 && is_per_or_int(b.bc[0])) {
        vaw = rdju[IDX2(b, 2, j)] / diu[IDX2(b, 2, j)] * dk[k - 1];
        vap = vap + vaw;
    }
    if (i == ni && !is_per_or_int(b.bc[1])) { vap = vap - vae; vae = 0.; }
    if (j == 2 && is_per_or_int(b.bc[2])) {
        vas = rdiv[IDX2(b, i, 2)] / djv[IDX2(b, i, 2)] * dk[k - 1];
        vap = vap + vas;
    }
    if (j == nj && !is_per_or_int(b.bc[3])) { vap = vap - van; van = 0.; }
    if (k == 2 && is_per_or_int(b.bc[4])) {
        val = didjp[IDX2(b, i, j)] / (rp[IDX2(b, i, j)] * dw[1]);
        vap = vap + val;
    }
    if (k == nk && !is_per_or_int(b.bc[5])) { vap = vap - var_; var_ = 0.; }
    ap[p] = vap; aw[p] = vaw; ae[p] = vae; as[p] = vas; an[p] = van; al[p] = val; ar[p] = var_;
    // starting surfaces (coeff_p_block.F:147-178)
    if (i == 2) ae[p - 1] = 0.;
    if (j == 2) an[p - b.n[0]] = 0.;
    if (k == 2) ar[p - (long)b.n[0] * b.n[1]] = 0.;
}

// ------------------------------------------------------------------- sour_p
// code/sour_p_block.F:161-241; every face flux of the running-flux loops is
// recomputed from the same operands, so the values are identical.
// ddtime = 2 / (3 dtime) * 0.5, cdtime = 2 / (3 dtime), rdtime = 1 / dtime,
// formed once on the host (the same IEEE operations): GB300's FP64 pipe
// made the three divisions per point the larger part of the kernel
__global__ void k_sour_p(const BlkDev *__restrict__ blk, double ddtime, double cdtime, double rdtime,
                         const double *__restrict__ rdiv, const double *__restrict__ rdju,
                         const double *__restrict__ didjp, const double *__restrict__ dkp,
                         const double *__restrict__ rdidjp, const double *__restrict__ dkw,
                         const double *__restrict__ u, const double *__restrict__ v,
                         const double *__restrict__ w, const double *__restrict__ rho,
                         const double *__restrict__ rhonp1, double *__restrict__ drhodt,
                         double *__restrict__ s, double *__restrict__ srhot,
                         double *__restrict__ srhoux)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long p = decode_interior(b, q, i, j, k);
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    double dkpk = dkp[b.off1k + k - 1];
    double gwf = rdju[IDX2(b, i, j)] * dkpk * (rhonp1[p] + rhonp1[p - 1]) * u[p];
    double gef = rdju[IDX2(b, i + 1, j)] * dkpk * (rhonp1[p] + rhonp1[p + 1]) * u[p + 1];
    double gsf = rdiv[IDX2(b, i, j)] * dkpk * (rhonp1[p] + rhonp1[p - jo]) * v[p];
    double gnf = rdiv[IDX2(b, i, j + 1)] * dkpk * (rhonp1[p] + rhonp1[p + jo]) * v[p + jo];
    double crf = didjp[IDX2(b, i, j)];
    double glf = crf * (rhonp1[p] + rhonp1[p - ko]) * w[p];
    double grf = crf * (rhonp1[p] + rhonp1[p + ko]) * w[p + ko];
    double sv = -ddtime * (gef - gwf + gnf - gsf + grf - glf);
    srhoux[p] = -ddtime * (gef - gwf + gnf - gsf + grf - glf);
    double vol = rdidjp[IDX2(b, i, j)] * dkw[b.off1k + k - 1];
    double dr = (rhonp1[p] - rho[p]) * rdtime;
    drhodt[p] = dr;
    s[p] = sv - cdtime * dr * vol;
    srhot[p] = -cdtime * dr * vol;
}

// -------------------------------------------------------------------- norms
// code/norms_block.F:443-467 per point; per-CTA partial sums of res^2,
// rhs^2, err^2, var^2 (deterministic order), finished by k_norms_final.
__global__ void k_norms(const BlkDev *__restrict__ blk, const double *__restrict__ ap,
                        const double *__restrict__ aw, const double *__restrict__ ae,
                        const double *__restrict__ as, const double *__restrict__ an,
                        const double *__restrict__ al, const double *__restrict__ ar,
                        const double *__restrict__ x, const double *__restrict__ bb,
                        double *__restrict__ residu, double *__restrict__ partial)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    double v[4] = {0., 0., 0., 0.};
    if (q < b.ncell) {
        int i, j, k;
        long p = decode_interior(b, q, i, j, k);
        long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
        double rhs = bb[p];
        double var = x[p];
        double res = bb[p] - ap[p] * var + aw[p] * x[p - 1] + ae[p] * x[p + 1] +
                     as[p] * x[p - jo] + an[p] * x[p + jo] + al[p] * x[p - ko] +
                     ar[p] * x[p + ko];
        double err = res / ap[p];
        v[0] = res * res;
        v[1] = rhs * rhs;
        v[2] = err * err;
        v[3] = var * var;
        residu[p] = res;
    }
    block_reduce_store<4>(v, partial + 4 * (blockIdx.y * (long)gridDim.x + blockIdx.x));
}

// Sum nparts partial vectors of width nv in a fixed order; out[0..nv) =
// sqrt(sum * rnpts), out[nv..2nv) = raw sums.  A zero last norm becomes 1
// (code/norms.F:398, code/sporlx.F:176).
__global__ void k_norms_final(const double *__restrict__ partial, long nparts, int nv,
                              double rnpts, double *__restrict__ out)
{
    double v[4] = {0., 0., 0., 0.};
    for (long t = threadIdx.x; t < nparts; t += blockDim.x)
        for (int c = 0; c < nv; c++) v[c] += partial[t * nv + c];
    __shared__ double res[4];
    block_reduce_store<4>(v, res);
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int c = 0; c < nv; c++) {
            out[nv + c] = res[c];
            out[c] = sqrt(res[c] * rnpts);
        }
        if (out[nv - 1] == 0.) out[nv - 1] = 1.;
    }
}

// --------------------------------------------------------- lexicographic SOR
// code/sporlx.F:211-275.  In every pass the point order is ascending in all
// three axes, so a point reads updated values at its -1 neighbours and old
// values at its +1 neighbours.  All points of one hyperplane i+j+k = s are
// therefore independent, and sweeping s upward reproduces the reference's
// result exactly.  `dir` (1, 2, 3) selects the operand order of the pass
// (sporlx.F:124-136).  With want_norm, the per-point terms of resnrm,
// errnrm, varnrm are stored for a later deterministic reduction.
__global__ void k_lex_wave(const BlkDev *__restrict__ blk, int s, int dir, double omega,
                           const double *__restrict__ ap, const double *__restrict__ aw,
                           const double *__restrict__ ae, const double *__restrict__ as,
                           const double *__restrict__ an, const double *__restrict__ al,
                           const double *__restrict__ ar, double *__restrict__ f,
                           const double *__restrict__ src, double *__restrict__ nrm3,
                           int want_norm)
{
    const BlkDev b = blk[blockIdx.y];
    int nj = b.n[1] - 2, nk = b.n[2] - 2;
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)nj * nk) return;
    int k = (int)(q / nj) + 2;
    int j = (int)(q - (long)(k - 2) * nj) + 2;
    int i = s - j - k;
    if (i < 2 || i > b.n[0] - 1) return;
    long p = IDX3(b, i, j, k);
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    double f_old = f[p];
    double dx;
    if (dir == 1)
        dx = (src[p] + aw[p] * f[p - 1] + ae[p] * f[p + 1] + as[p] * f[p - jo] +
              an[p] * f[p + jo] + al[p] * f[p - ko] + ar[p] * f[p + ko]) / ap[p] - f_old;
    else if (dir == 2)
        dx = (src[p] + as[p] * f[p - jo] + an[p] * f[p + jo] + aw[p] * f[p - 1] +
              ae[p] * f[p + 1] + al[p] * f[p - ko] + ar[p] * f[p + ko]) / ap[p] - f_old;
    else
        dx = (src[p] + al[p] * f[p - ko] + ar[p] * f[p + ko] + aw[p] * f[p - 1] +
              ae[p] * f[p + 1] + as[p] * f[p - jo] + an[p] * f[p + jo]) / ap[p] - f_old;
    double fn = f_old + omega * dx;
    f[p] = fn;
    if (want_norm) {
        dx = fn - f_old;
        double res = dx * ap[p];
        nrm3[3 * p + 0] = res * res;
        nrm3[3 * p + 1] = dx * dx;
        nrm3[3 * p + 2] = fn * fn;
    }
}

// partial sums of the stored per-point SOR norm terms
__global__ void k_lex_norm_partial(const BlkDev *__restrict__ blk, const double *__restrict__ nrm3,
                                   double *__restrict__ partial)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    double v[3] = {0., 0., 0.};
    if (q < b.ncell) {
        int i, j, k;
        long p = decode_interior(b, q, i, j, k);
        v[0] = nrm3[3 * p];
        v[1] = nrm3[3 * p + 1];
        v[2] = nrm3[3 * p + 2];
    }
    block_reduce_store<3>(v, partial + 3 * (blockIdx.y * (long)gridDim.x + blockIdx.x));
}

// -------------------------------------------------------------- restriction
// code/rest_block.F:98-144, one coarse interior point per thread.
__global__ void k_restrict(const BlkDev *__restrict__ bc_, const BlkDev *__restrict__ bf_,
                           const double *__restrict__ ff, double *__restrict__ fc)
{
    const BlkDev c = bc_[blockIdx.y], fb = bf_[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= c.ncell) return;
    int i, j, k;
    long pc = decode_interior(c, q, i, j, k);
    long jof = fb.n[0], kof = (long)fb.n[0] * fb.n[1];
    double fac = 1.0;
    long iinc, jinc, kinc;
    if (fb.mult[0] == 1) { iinc = 0; fac = 0.5 * fac; } else iinc = -1;
    if (fb.mult[1] == 1) { jinc = 0; fac = 0.5 * fac; } else jinc = -jof;
    if (fb.mult[2] == 1) { kinc = 0; fac = 0.5 * fac; } else kinc = -kof;
    long pf = fb.off3 + (fb.mult[0] * i - 2) + jof * (fb.mult[1] * j - 2) + kof * (fb.mult[2] * k - 2);
    fc[pc] = fac * (ff[pf] + ff[pf + iinc] + ff[pf + jinc] + ff[pf + iinc + jinc] + ff[pf + kinc] +
                    ff[pf + iinc + kinc] + ff[pf + jinc + kinc] + ff[pf + iinc + jinc + kinc]);
}

// ------------------------------------------------------------- prolongation
// code/prol_block.F:325-357: on every non-interface side the coarse ghost
// plane takes the value of its interior neighbour, sides 1..6 in turn (one
// CTA per block so the side order is kept).
__global__ void k_prol_ghost(const BlkDev *__restrict__ blk, double *__restrict__ f)
{
    const BlkDev b = blk[blockIdx.x];
    const int cyc1[2][4] = {{0, 2, 1, 1}, {0, 3, 3, 2}};
    long st[4] = {0, 1, b.n[0], (long)b.n[0] * b.n[1]};
    int nn[4] = {0, b.n[0], b.n[1], b.n[2]};
    for (int s = 1; s <= 6; s++) {
        if (b.bc[s - 1] != LES_BCT_INTERFACE_D) {
            int d1 = (s + 1) / 2, d2 = cyc1[0][d1], d3 = cyc1[1][d1];
            long base = (s % 2 == 1) ? 0 : st[d1] * (nn[d1] - 1);
            long inext = (s % 2 == 1) ? st[d1] : -st[d1];
            long n = (long)nn[d2] * nn[d3];
            for (long q = threadIdx.x; q < n; q += blockDim.x) {
                long kk = q / nn[d2], jj = q - kk * nn[d2];
                long p = b.off3 + base + st[d2] * jj + st[d3] * kk;
                f[p] = f[p + inext];
            }
        }
        __syncthreads();
    }
}

// code/prol_block.F:363-469.  Each fine point receives exactly one trilinear
// contribution (from coarse cell ((i+1)/2, (j+1)/2, (k+1)/2)), summed from
// zero in the reference's operand order; the correction is added on the
// interior and on interface ghost planes.
__global__ void k_prol_fine(const BlkDev *__restrict__ bc_, const BlkDev *__restrict__ bf_,
                            const double *__restrict__ fcv, double *__restrict__ ff)
{
    const BlkDev c = bc_[blockIdx.y], fb = bf_[blockIdx.y];
    int is = fb.bc[0] == LES_BCT_INTERFACE_D ? 1 : 2;
    int ie = fb.bc[1] == LES_BCT_INTERFACE_D ? fb.n[0] : fb.n[0] - 1;
    int js = fb.bc[2] == LES_BCT_INTERFACE_D ? 1 : 2;
    int je = fb.bc[3] == LES_BCT_INTERFACE_D ? fb.n[1] : fb.n[1] - 1;
    int ks = fb.bc[4] == LES_BCT_INTERFACE_D ? 1 : 2;
    int ke = fb.bc[5] == LES_BCT_INTERFACE_D ? fb.n[2] : fb.n[2] - 1;
    int ni = ie - is + 1, nj = je - js + 1, nk = ke - ks + 1;
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)ni * nj * nk) return;
    long t = q / ni;
    int i = (int)(q - t * ni) + is;
    int k = (int)(t / nj) + ks;
    int j = (int)(t - (long)(k - ks) * nj) + js;
    const double w[4] = {0.421875, 0.140625, 0.046875, 0.015625};
    int ic, jc, kc, a, bb, cc;
    if (fb.mult[0] == 2) { ic = (i + 1) / 2; a = (i + 1) & 1; } else { ic = i; a = 0; }
    if (fb.mult[1] == 2) { jc = (j + 1) / 2; bb = (j + 1) & 1; } else { jc = j; bb = 0; }
    if (fb.mult[2] == 2) { kc = (k + 1) / 2; cc = (k + 1) & 1; } else { kc = k; cc = 0; }
    long joc = c.n[0], koc = (long)c.n[0] * c.n[1];
    long pc = c.off3 + (ic - 1) + joc * (jc - 1) + koc * (kc - 1);
    // source corners in the reference's term order: P, E, N, R, NE, NR, ER, ENR
    const int sx[8] = {0, 1, 0, 0, 1, 0, 1, 1};
    const int sy[8] = {0, 0, 1, 0, 1, 1, 0, 1};
    const int sz[8] = {0, 0, 0, 1, 0, 1, 1, 1};
    double cr = 0.;
#pragma unroll
    for (int m = 0; m < 8; m++) {
        int h = (sx[m] != a) + (sy[m] != bb) + (sz[m] != cc);
        cr = cr + w[h] * fcv[pc + sx[m] + joc * sy[m] + koc * sz[m]];
    }
    long pf = fb.off3 + (i - 1) + (long)fb.n[0] * ((j - 1) + (long)fb.n[1] * (k - 1));
    ff[pf] = ff[pf] + cr;
}

// ----------------------------------------------------------------- extrap_p
// code/extrap_p_block.F:335-366: ghost plane := adjacent interior plane on
// every side that is neither periodic nor interface, sides 1..6 in turn.
// side s of every block (one launch per side, the sides in the reference's
// order: an edge point two sides share takes the later side's value)
__global__ void k_extrap_p(const BlkDev *__restrict__ blk, int s, double *__restrict__ p)
{
    pdl_wait();
    pdl_trigger();
    const BlkDev b = blk[blockIdx.y];
    if (is_per_or_int(b.bc[s - 1])) return;
    const int co[2][4] = {{0, 2, 1, 1}, {0, 3, 3, 2}};
    long st[4] = {0, 1, b.n[0], (long)b.n[0] * b.n[1]};
    int nn[4] = {0, b.n[0], b.n[1], b.n[2]};
    int d1 = (s + 1) / 2, d2 = co[0][d1], d3 = co[1][d1];
    long base = (s % 2 == 1) ? 0 : st[d1] * (nn[d1] - 1);
    long io1 = (s % 2 == 0) ? -st[d1] : st[d1];
    long n = (long)nn[d2] * nn[d3];
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        long kk = q / nn[d2], jj = q - kk * nn[d2];
        long ijk = b.off3 + base + st[d2] * jj + st[d3] * kk;
        p[ijk] = p[ijk + io1];
    }
}

// ----------------------------------------------------------- p_ref_subtract
// code/p_ref_subtract.F:39-93: the value at (2,2,2) of block 1 is taken
// first, then subtracted everywhere (ghosts included).
__global__ void k_pref_get(const BlkDev *__restrict__ blk, const double *__restrict__ p,
                           double *__restrict__ pref)
{
    pdl_wait();
    pdl_trigger();
    const BlkDev b = blk[0];
    pref[0] = p[IDX3(b, 2, 2, 2)];
}

__global__ void k_pref_sub(double *__restrict__ p, long n, const double *__restrict__ pref)
{
    pdl_wait();
    pdl_trigger();
    double r = pref[0];
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        p[q] = p[q] - r;
}

// ------------------------------------------------------------------ uvw_adv
// code/uvw_adv_block.F:199-269 for one component; the loop start is 3 on
// a non-periodic, non-interface inflow side (code/set_loop_bound.F:328-345).
__global__ void k_uvw_adv(const BlkDev *__restrict__ blk, int ivar, double dtime,
                          const double *__restrict__ dg, const double *__restrict__ rp,
                          const double *__restrict__ dkw, double *__restrict__ u,
                          const double *__restrict__ u_int, const double *__restrict__ rho,
                          const double *__restrict__ p)
{
    pdl_wait();
    pdl_trigger();
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long ijk = decode_interior(b, q, i, j, k);
    int istr = (ivar == 1 && !is_per_or_int(b.bc[0])) ? 3 : 2;
    int jstr = (ivar == 2 && !is_per_or_int(b.bc[2])) ? 3 : 2;
    int kstr = (ivar == 3 && !is_per_or_int(b.bc[4])) ? 3 : 2;
    if (ivar == 3) istr = jstr; // uvw_adv_block.F:255 starts the W i-loop at jstr
    if (i < istr || j < jstr || k < kstr) return;
    double ddtime = 1.5 * dtime;
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    double dpdi, rhou;
    if (ivar != 3) {
        long ijkw = ijk - (ivar == 1 ? 1 : jo);
        dpdi = (p[ijk] - p[ijkw]) / dg[IDX2(b, i, j)];
        rhou = 0.5 * (rho[ijk] + rho[ijkw]);
    } else {
        long ijkl = ijk - ko;
        dpdi = (p[ijk] - p[ijkl]) / (rp[IDX2(b, i, j)] * dkw[b.off1k + k - 1]);
        rhou = 0.5 * (rho[ijk] + rho[ijkl]);
    }
    u[ijk] = u_int[ijk] - ddtime * dpdi / rhou;
}

// The projection with FP32 arithmetic (the mixed path with FP32 physics):
// the pressure difference is taken in FP64 and rounded once, the correction
// dt grad p / rho is formed in FP32 and subtracted from the FP64 u_int in
// FP64, so u keeps u_int's precision and the correction carries FP32's
// (GB300 issues FP64 divisions slowly; this kernel has none).
__global__ void k_uvw_adv_f32(const BlkDev *__restrict__ blk, int ivar, float dtime,
                              const double *__restrict__ dg, const double *__restrict__ rp,
                              const double *__restrict__ dkw, double *__restrict__ u,
                              const double *__restrict__ u_int, const double *__restrict__ rho,
                              const double *__restrict__ p)
{
    pdl_wait();
    pdl_trigger();
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long ijk = decode_interior(b, q, i, j, k);
    int istr = (ivar == 1 && !is_per_or_int(b.bc[0])) ? 3 : 2;
    int jstr = (ivar == 2 && !is_per_or_int(b.bc[2])) ? 3 : 2;
    int kstr = (ivar == 3 && !is_per_or_int(b.bc[4])) ? 3 : 2;
    if (ivar == 3) istr = jstr;
    if (i < istr || j < jstr || k < kstr) return;
    const long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    const long nb = ijk - (ivar == 1 ? 1 : ivar == 2 ? jo : ko);
    const float dp = (float)(p[ijk] - p[nb]);
    const float h = ivar != 3 ? (float)dg[IDX2(b, i, j)]
                              : (float)rp[IDX2(b, i, j)] * (float)dkw[b.off1k + k - 1];
    const float rhou = 0.5f * (float)(rho[ijk] + rho[nb]);
    const float corr = 1.5f * dtime * (dp / h) / rhou;
    u[ijk] = u_int[ijk] - (double)corr;
}

// ------------------------------------------------- density and slip faces
// code/swap_rhos_block.F:438-451
__global__ void k_swap_rhos(double *__restrict__ rho, const double *__restrict__ rhonp1,
                            double *__restrict__ rhonm1, long n)
{
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        double r = rho[q];
        rhonm1[q] = r;
        rho[q] = rhonp1[q];
    }
}

// code/search_lib_block.F:374-399
__global__ void k_search_lib(double *__restrict__ sc1, double *__restrict__ rhonp1,
                             const double *__restrict__ rho, double alpha, double rholo,
                             double rhohi, long n)
{
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        double f = sc1[q];
        double rho_mix = 1.0 / (f / rhohi + (1.0 - f) / rholo);
        if (f > 1.0) rho_mix = rhohi;
        if (f < 0.0) rho_mix = rholo;
        double rn = alpha * rho[q] + (1.0 - alpha) * rho_mix;
        rhonp1[q] = rn;
        f = (f * rho[q]) / rn;
        if (f > 1.0) f = 1.0;
        sc1[q] = f;
    }
}

// search_lib with FP32 arithmetic (the mixed path with FP32 physics): the
// mixing law and the conservative scalar rescaling of k_search_lib, FP64
// fields rounded once on load and once on store.
__global__ void k_search_lib_f32(double *__restrict__ sc1, double *__restrict__ rhonp1,
                                 const double *__restrict__ rho, float alpha, float rholo, float rhohi,
                                 long n)
{
    const float irhohi = 1.0f / rhohi, irholo = 1.0f / rholo;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        float f = (float)sc1[q];
        const float r = (float)rho[q];
        float rho_mix = 1.0f / (f * irhohi + (1.0f - f) * irholo);
        if (f > 1.0f) rho_mix = rhohi;
        if (f < 0.0f) rho_mix = rholo;
        const float rn = alpha * r + (1.0f - alpha) * rho_mix;
        rhonp1[q] = (double)rn;
        f = (f * r) / rn;
        if (f > 1.0f) f = 1.0f;
        sc1[q] = (double)f;
    }
}

// code/slipbc.F:80-190 for the j sides (TRACTION and ZERO_GRAD); one
// thread per (i, k) of the side, i = 1..nip1, k = 2..nkp1-1.
__global__ void k_slipbc(const BlkDev *__restrict__ blk, double dtime,
                         const double *__restrict__ djp, double *__restrict__ u,
                         double *__restrict__ v, const double *__restrict__ v_int,
                         double *__restrict__ w, double *__restrict__ sc1,
                         double *__restrict__ rho, const double *__restrict__ p)
{
    const BlkDev b = blk[blockIdx.y];
    int nip1 = b.n[0], njp1 = b.n[1], nkp1 = b.n[2];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)nip1 * (nkp1 - 2)) return;
    int i = (int)(q % nip1) + 1;
    int k = (int)(q / nip1) + 2;
    long jo = nip1;
    double ddtime = 1.5 * dtime;
    // the four passes of slipbc_block, in source order
    if (b.bc[2] == LES_BCT_TRACTION_D) {
        long ijk = IDX3(b, i, 2, k), ijks = ijk - jo;
        sc1[ijks] = sc1[ijk];
        rho[ijks] = rho[ijk];
        double rhou = 0.5 * (rho[ijk] + rho[ijks]);
        u[ijks] = u[ijk];
        v[ijk] = v_int[ijk] - ddtime * ((2.0 * p[ijk] - 2.0 * 0.0) / djp[IDX2(b, i, 1)]) / rhou;
        v[ijks] = v[ijk];
        w[ijks] = w[ijk];
    }
    if (b.bc[3] == LES_BCT_TRACTION_D) {
        long ijk = IDX3(b, i, njp1 - 1, k), ijkn = ijk + jo;
        sc1[ijkn] = sc1[ijk];
        rho[ijkn] = rho[ijk];
        double rhou = 0.5 * (rho[ijk] + rho[ijkn]);
        u[ijkn] = u[ijk];
        v[ijkn] = v_int[ijkn] - ddtime * ((-2.0 * p[ijk] + 2.0 * 0.0) / djp[IDX2(b, i, njp1 - 1)]) / rhou;
        w[ijkn] = w[ijk];
    }
    if (b.bc[2] == LES_BCT_ZERO_GRAD_D) {
        long ijk = IDX3(b, i, 2, k), ijks = ijk - jo;
        sc1[ijks] = sc1[ijk];
        rho[ijks] = rho[ijk];
        u[ijks] = u[ijk];
        v[ijk] = 0.0;
        v[ijks] = 0.0;
        w[ijks] = w[ijk];
    }
    if (b.bc[3] == LES_BCT_ZERO_GRAD_D) {
        long ijk = IDX3(b, i, njp1 - 1, k), ijkn = ijk + jo;
        sc1[ijkn] = sc1[ijk];
        rho[ijkn] = rho[ijk];
        u[ijkn] = u[ijk];
        v[ijkn] = 0.0;
        w[ijkn] = w[ijk];
    }
}

// ================================================================ launchers
namespace les {

static inline unsigned nblk(long n, int t) { return (unsigned)((n + t - 1) / t); }

void launch_halo(const FaceDev *faces, int nface, long maxface, double *var, double *work,
                 cudaStream_t st)
{
    if (nface == 0) return;
    unsigned gx = nblk(maxface, 256);
    if (gx > 64) gx = 64;
    launch_pdl(k_halo_pack, dim3(gx, nface), dim3(256), 0, st, faces, var, work);
    launch_pdl(k_halo_unpack, dim3(gx, nface), dim3(256), 0, st, faces, var, work);
    count_launch(2);
}

void launch_coeff_p(const BlkDev *blk, int nb, long maxcell, const double *const *m,
                    const double *dkp, const double *dkw, double *const *a, cudaStream_t st)
{
    // m: diu, djv, rdiv, rdju, didjp, rp ; a: ap, aw, ae, as, an, al, ar
    k_coeff_p<<<dim3(nblk(maxcell, 128), nb), 128, 0, st>>>(blk, m[0], m[1], m[2], m[3], m[4], m[5],
                                                          dkp, dkw, a[0], a[1], a[2], a[3], a[4],
                                                          a[5], a[6]);
    count_launch(1);
}

void launch_sour_p(const BlkDev *blk, int nb, long maxcell, double dtime, const double *rdiv,
                   const double *rdju, const double *didjp, const double *dkp,
                   const double *rdidjp, const double *dkw, const double *u, const double *v,
                   const double *w, const double *rho, const double *rhonp1, double *drhodt,
                   double *s, double *srhot, double *srhoux, cudaStream_t st)
{
    const double cdtime = 2.0 / (3.0 * dtime), ddtime = cdtime * 0.5, rdtime = 1.0 / dtime;
    k_sour_p<<<dim3(nblk(maxcell, 128), nb), 128, 0, st>>>(blk, ddtime, cdtime, rdtime, rdiv, rdju, didjp, dkp,
                                                         rdidjp, dkw, u, v, w, rho, rhonp1, drhodt, s, srhot,
                                                         srhoux);
    count_launch(1);
}

long norms_parts(int nb, long maxcell) { return (long)nblk(maxcell, 256) * nb; }

void launch_norms(const BlkDev *blk, int nb, long maxcell, const double *const *a, const double *x,
                  const double *b, double *residu, double *partial, double rnpts, double *out,
                  cudaStream_t st)
{
    unsigned gx = nblk(maxcell, 256);
    k_norms<<<dim3(gx, nb), 256, 0, st>>>(blk, a[0], a[1], a[2], a[3], a[4], a[5], a[6], x, b, residu,
                                         partial);
    k_norms_final<<<1, 256, 0, st>>>(partial, (long)gx * nb, 4, rnpts, out);
    count_launch(2);
}

void launch_lex_pass(const BlkDev *blk, int nb, int maxjk, int smin, int smax, int dir, double omega,
                     const double *const *a, double *f, const double *src, double *nrm3,
                     int want_norm, cudaStream_t st)
{
    unsigned gx = nblk(maxjk, 128);
    for (int s = smin; s <= smax; s++)
        k_lex_wave<<<dim3(gx, nb), 128, 0, st>>>(blk, s, dir, omega, a[0], a[1], a[2], a[3], a[4], a[5],
                                                a[6], f, src, nrm3, want_norm);
    count_launch(smax - smin + 1);
}

void launch_lex_norm(const BlkDev *blk, int nb, long maxcell, const double *nrm3, double *partial,
                     double rnpts, double *out, cudaStream_t st)
{
    unsigned gx = nblk(maxcell, 256);
    k_lex_norm_partial<<<dim3(gx, nb), 256, 0, st>>>(blk, nrm3, partial);
    k_norms_final<<<1, 256, 0, st>>>(partial, (long)gx * nb, 3, rnpts, out);
    count_launch(2);
}

void launch_restrict(const BlkDev *bc, const BlkDev *bf, int nb, long maxcell_c, const double *ff,
                     double *fc, cudaStream_t st)
{
    k_restrict<<<dim3(nblk(maxcell_c, 128), nb), 128, 0, st>>>(bc, bf, ff, fc);
    count_launch(1);
}

void launch_prolong(const BlkDev *bc, const BlkDev *bf, int nb, long maxfine, double *f,
                    cudaStream_t st)
{
    k_prol_ghost<<<nb, 512, 0, st>>>(bc, f);
    k_prol_fine<<<dim3(nblk(maxfine, 128), nb), 128, 0, st>>>(bc, bf, f, f);
    count_launch(2);
}

void launch_extrap_p(const BlkDev *blk, int nb, double *p, cudaStream_t st)
{
    // a side of a block holds at most 64 k points in these grids; 64 CTAs of
    // 256 threads per block and side, grid-stride beyond
    for (int s = 1; s <= 6; s++) launch_pdl(k_extrap_p, dim3(64, nb), dim3(256), 0, st, blk, s, p);
    count_launch(6);
}

void launch_pref(const BlkDev *blk, double *p, long n, double *scratch, cudaStream_t st)
{
    launch_pdl(k_pref_get, dim3(1), dim3(1), 0, st, blk, p, scratch);
    const unsigned g = nblk(n, 256) > 2048 ? 2048 : nblk(n, 256);
    launch_pdl(k_pref_sub, dim3(g), dim3(256), 0, st, p, n, (const double *)scratch);
    count_launch(2);
}

void launch_uvw_adv(const BlkDev *blk, int nb, long maxcell, int ivar, double dtime,
                    const double *dg, const double *rp, const double *dkw, double *u,
                    const double *u_int, const double *rho, const double *p, bool f32, cudaStream_t st)
{
    if (f32)
        launch_pdl(k_uvw_adv_f32, dim3(nblk(maxcell, 256), nb), dim3(256), 0, st, blk, ivar, (float)dtime, dg, rp, dkw,
                   u, u_int, rho, p);
    else
        launch_pdl(k_uvw_adv, dim3(nblk(maxcell, 128), nb), dim3(128), 0, st, blk, ivar, dtime, dg, rp, dkw, u, u_int,
                   rho, p);
    count_launch(1);
}

void launch_swap_rhos(double *rho, const double *rhonp1, double *rhonm1, long n, cudaStream_t st)
{
    unsigned g = nblk(n, 256);
    k_swap_rhos<<<g > 4096 ? 4096 : g, 256, 0, st>>>(rho, rhonp1, rhonm1, n);
    count_launch(1);
}

void launch_search_lib(double *sc1, double *rhonp1, const double *rho, double alpha, double rholo,
                       double rhohi, long n, bool f32, cudaStream_t st)
{
    unsigned g = nblk(n, 256);
    if (f32)
        k_search_lib_f32<<<g > 4096 ? 4096 : g, 256, 0, st>>>(sc1, rhonp1, rho, (float)alpha, (float)rholo,
                                                             (float)rhohi, n);
    else
        k_search_lib<<<g > 4096 ? 4096 : g, 256, 0, st>>>(sc1, rhonp1, rho, alpha, rholo, rhohi, n);
    count_launch(1);
}

void launch_slipbc(const BlkDev *blk, int nb, long maxik, double dtime, const double *djp,
                   double *u, double *v, const double *v_int, double *w, double *sc1,
                   double *rho, const double *p, cudaStream_t st)
{
    k_slipbc<<<dim3(nblk(maxik, 128), nb), 128, 0, st>>>(blk, dtime, djp, u, v, v_int, w, sc1, rho, p);
    count_launch(1);
}

} // namespace les
