// lester_outflow.cu -- convective outflow and fixed inflow sides (C ABI):
//   lester_conv_exitbc   code/conv_exitbc.F:21
//   lester_mass_change   code/mass_change.F:6
//   lester_fixed_inlet   code/fixed_inlet.F:5
//   lester_gpu_set_inlet (the inlet blocks inlet1..inlet4 of COMMON and the
//                         profiles read_profile reads from inflowbc.3d)
//
// conv_exitbc keeps SAVEd values between calls (conv_exitbc.F:78): the
// per-side outflow mass flux and rho-weighted area of step n, and the
// inflow/outflow sums accumulated over the calls iva = u, v, w.  They live
// in a small device array, so a step's calls chain on the stream with no
// host round trip; MPI_ALLREDUCE sums become sums over the sides in (block,
// side) order.
#include <cstring>
#include <vector>

#include "kernels.h"
#include "lester_ctx.h"

namespace les {

static bool per_int_bc(int bc) { return bc == LES_BCT_PERIODIC || bc == LES_BCT_INTERFACE; }

int ensure_sides(Ctx &c)
{
    if (c.sides_built) return 0;
    std::vector<SideJob> v;
    for (int b = 1; b <= c.g.numbl; b++)
        for (int s = 1; s <= 6; s++) {
            int bc = c.g.bl_bc[b - 1][s - 1];
            if (bc != LES_BCT_CONVECTIVE && bc != LES_BCT_FIXED) continue;
            if (bc == LES_BCT_CONVECTIVE && s == 5)
                return set_err(LES_ERR_GEOM,
                               "block %d: a convective low-z side reads below the block at k = 0 "
                               "(conv_exitbc1_block.F:110-122); not supported", b);
            SideJob J;
            memset(&J, 0, sizeof J);
            J.blk = b - 1;
            J.side = s;
            J.d1 = (s + 1) / 2;
            J.conv = bc == LES_BCT_CONVECTIVE;
            const int *n = c.lv[1].n[b];
            for (int a = 0; a < 3; a++) J.n[a] = n[a];
            J.off3 = c.lv[1].off3[b];
            J.off2 = c.lv[1].off2[b];
            J.off1k = c.lv[1].off1k[b];
            const int *bcb = c.g.bl_bc[b - 1];
            for (int iv = 1; iv <= 3; iv++) {
                // set_loop_bound(iv, 1, 1, iblk, iblk, 1, ijkse) at level 1
                int *se = J.bnd[iv];
                se[0] = (iv == 1 && !per_int_bc(bcb[0])) ? 3 : 2;
                se[1] = n[0] - 1;
                se[2] = (iv == 2 && !per_int_bc(bcb[2])) ? 3 : 2;
                se[3] = n[1] - 1;
                se[4] = (iv == 3 && !per_int_bc(bcb[4])) ? 3 : 2;
                se[5] = n[2] - 1;
            }
            const int *sd = J.bnd[J.d1];
            J.plane = (s % 2 == 1) ? sd[2 * J.d1 - 2] - 1 : sd[2 * J.d1 - 1] + 1;
            v.push_back(J);
        }
    c.sides = v;
    if (!v.empty()) {
        LES_CUDA(cudaMalloc(&c.d_sides, sizeof(SideJob) * v.size()));
        LES_CUDA(cudaMemcpy(c.d_sides, v.data(), sizeof(SideJob) * v.size(), cudaMemcpyHostToDevice));
        LES_CUDA(cudaMalloc(&c.d_sideout, sizeof(double) * 3 * v.size()));
    }
    LES_CUDA(cudaMalloc(&c.d_exit, sizeof(double) * EX_N));
    LES_CUDA(cudaMemset(c.d_exit, 0, sizeof(double) * EX_N));
    c.sides_built = true;
    return 0;
}

bool has_convective(const Ctx &c)
{
    for (const SideJob &J : c.sides)
        if (J.conv) return true;
    return false;
}

enum { X_DIP, X_DIU, X_DIX, X_DJP, X_DJV, X_DJX, X_RDIV, X_RDJU, X_DIDJP, X_RP, X_RU, X_RV, X_N };

// one conv_exitbc call on device arrays; m[] the 2-D metrics of X_*
int exit_task(Ctx &c, int task, int iva, const double *rho, const double *rhonp1, double *u, double *v,
              double *w, double *u_int, double *v_int, double *w_int, double *hu, double *hv, double *hw,
              const double *const *m, const double *dkp, const double *dkw, const double *rdidjp)
{
    int r;
    if ((r = ensure_sides(c))) return r;
    if (!has_convective(c)) return 0;  // conv_exitbc.F:92-115
    const int nj = (int)c.sides.size();
    cudaStream_t st = c.stream;
    const double *ru = m[X_RDJU], *rv = m[X_RDIV], *dd = m[X_DIDJP];
    if (task == 1 && iva == 1) {
        launch_side_flux(c.d_sides, nj, 0, 1, u, v, w, rhonp1, ru, rv, dd, dkp, c.d_sideout, st);
        launch_side_combine(c.d_sides, nj, c.d_sideout, 0, c.d_exit, st);
    }
    if (iva == 1) launch_side_combine(c.d_sides, nj, c.d_sideout, 3, c.d_exit, st);
    const double *fu = task == 1 ? u_int : u, *fv = task == 1 ? v_int : v, *fw = task == 1 ? w_int : w;
    // inflow sums (fixed sides; only the side's own axis contributes)
    if (iva >= 1 && iva <= 3) {
        launch_side_flux(c.d_sides, nj, iva, 0, fu, fv, fw, rhonp1, ru, rv, dd, dkp, c.d_sideout, st);
        launch_side_combine(c.d_sides, nj, c.d_sideout, 1, c.d_exit, st);
        // the exit planes of this variable (conv_exitbc.F:262-338, 437-497)
        ExitMetrics M;
        memset(&M, 0, sizeof M);
        M.dm[1] = m[iva == 1 ? X_DIP : iva == 2 ? X_DIX : X_DIU];
        M.dm[2] = m[iva == 1 ? X_DJX : iva == 2 ? X_DJP : X_DJV];
        M.dm[3] = m[X_DJX];
        M.rm[1] = M.rm[2] = m[X_RP];
        M.rm[3] = m[iva == 1 ? X_RU : iva == 2 ? X_RV : X_RP];
        M.km[1] = M.km[2] = dkp;
        M.km[3] = iva == 3 ? dkp : dkw;
        double *vel = iva == 1 ? u : iva == 2 ? v : w;
        double *vint = iva == 1 ? u_int : iva == 2 ? v_int : w_int;
        double *hn = iva == 1 ? hu : iva == 2 ? hv : hw;
        launch_exit_update(c.d_sides, nj, task, iva, M, vel, vint, rho, rhonp1, hn, c.c.dtime, c.d_exit, st);
        // outflow sums after the update
        launch_side_flux(c.d_sides, nj, iva, 1, fu, fv, fw, rhonp1, ru, rv, dd, dkp, c.d_sideout, st);
        launch_side_combine(c.d_sides, nj, c.d_sideout, 2, c.d_exit, st);
    }
    if (iva == 3 && task == 1) {
        LevelGeom &L = c.lv[1];
        launch_mass_change(L.d_blk, c.g.numbl, L.maxcell, c.c.dtime, rho, rhonp1, rdidjp, dkw, c.d_partial,
                           c.d_exit + EX_MCHG, st);
        double *ints[3] = {u_int, v_int, w_int};
        for (int iv = 1; iv <= 3; iv++) launch_exit_scale(c.d_sides, nj, iv, ints[iv - 1], c.d_exit, st);
    }
    LES_CUDA(cudaGetLastError());
    return 0;
}

// fixed_inlet on device arrays with device profiles
int inlet_task(Ctx &c, const double *uprof, const double *vprof, unsigned long long seed, int step, double *u,
               double *v, double *w, double *sc1, double *rho, double *u_int, double *v_int, double *w_int)
{
    for (int q = 0; q < 4; q++) {
        int b = c.inlet[q];
        if (b < 1 || b > c.g.numbl) continue;
        // every block listed more than once takes its last slot, as the
        // reference's if-chain (fixed_inlet.F:87-131) lets the last match win
        int which = 0;
        for (int q2 = 0; q2 < 4; q2++)
            if (c.inlet[q2] == b) which = q2 + 1;
        if (which != q + 1) continue;
        const int *n = c.lv[1].n[b];
        int nj = n[1] - 1;
        long need = (long)n[1] + (long)(which - 1) * (nj - 1);
        long need_amp = which <= 2 ? 3 : 4L * (nj - 2);
        if (std::max(need, need_amp) > c.nprof)
            return set_err(LES_ERR_ARG, "inlet block %d needs %ld profile values, %d given", b,
                           std::max(need, need_amp), c.nprof);
        // inside the whole-step graph's capture the step comes from device
        // memory (d_step[1], written before each replay)
        launch_fixed_inlet(c.lv[1].d_blk, b - 1, which, n[1] * n[2], uprof, vprof, seed, step,
                           c.capturing ? c.d_step + 1 : nullptr, c.c.rholo,
                           c.c.rhohi, u, v, w, sc1, rho, u_int, v_int, w_int, c.stream);
    }
    LES_CUDA(cudaGetLastError());
    return 0;
}

bool has_inlet(const Ctx &c) { return c.inlet[0] || c.inlet[1] || c.inlet[2] || c.inlet[3]; }

} // namespace les

using namespace les;

extern "C" {

int lester_conv_exitbc(const int *task, const int *iva, const double *rho, const double *rhonp1, double *u,
                       double *v, double *w, double *u_int, double *v_int, double *w_int, double *hu, double *hv,
                       double *hw, const double *dip, const double *diu, const double *dix, const double *djp,
                       const double *djv, const double *djx, const double *rdiv, const double *rdju,
                       const double *didjp, const double *rp, const double *ru, const double *rv,
                       const double *dkp, const double *dkw, const double *rdidjp)
{
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    if (!task || !iva || (*task != 1 && *task != 2) || *iva < 1 || *iva > 5)
        return set_err(LES_ERR_ARG, "conv_exitbc: task must be 1 or 2 and iva 1..5");
    int r;
    if ((r = ensure_sides(c))) return r;
    if (!has_convective(c)) return 0;
    Staging st(&c, __func__);
    const double *d3i[2];
    const double *in3[2] = {rho, rhonp1};
    for (int q = 0; q < 2; q++)
        if ((r = st.in(in3[q], c.tot_sg3, &d3i[q]))) return r;
    double *d3[9];
    double *io3[9] = {u, v, w, u_int, v_int, w_int, hu, hv, hw};
    for (int q = 0; q < 9; q++)
        if ((r = st.io(io3[q], c.tot_sg3, &d3[q]))) return r;
    const double *m[X_N];
    const double *mu[X_N] = {dip, diu, dix, djp, djv, djx, rdiv, rdju, didjp, rp, ru, rv};
    for (int q = 0; q < X_N; q++)
        if ((r = st.in(mu[q], c.tot2, &m[q]))) return r;
    const double *dk[3];
    if ((r = st.in(dkp, c.tot1k, &dk[0])) || (r = st.in(dkw, c.tot1k, &dk[1])) ||
        (r = st.in(rdidjp, c.tot2, &dk[2])))
        return r;
    if ((r = exit_task(c, *task, *iva, d3i[0], d3i[1], d3[0], d3[1], d3[2], d3[3], d3[4], d3[5], d3[6], d3[7],
                       d3[8], m, dk[0], dk[1], dk[2])))
        return r;
    return st.finish();
}

int lester_mass_change(const double *rho, const double *rhonp1, double *mass_chg, const double *rdidjp,
                       const double *dkw)
{
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    if (!mass_chg) return set_err(LES_ERR_ARG, "mass_change: NULL result");
    int r;
    if ((r = ensure_sides(c))) return r;
    Staging st(&c, __func__);
    const double *d[4];
    if ((r = st.in(rho, c.tot_sg3, &d[0])) || (r = st.in(rhonp1, c.tot_sg3, &d[1])) ||
        (r = st.in(rdidjp, c.tot2, &d[2])) || (r = st.in(dkw, c.tot1k, &d[3])))
        return r;
    LevelGeom &L = c.lv[1];
    launch_mass_change(L.d_blk, c.g.numbl, L.maxcell, c.c.dtime, d[0], d[1], d[2], d[3], c.d_partial,
                       c.d_exit + EX_MCHG, c.stream);
    LES_CUDA(cudaMemcpyAsync(c.h_small + 48, c.d_exit + EX_MCHG, sizeof(double), cudaMemcpyDeviceToHost,
                             c.stream));
    LES_CUDA(cudaStreamSynchronize(c.stream));
    *mass_chg = c.h_small[48];
    return st.finish();
}

int lester_gpu_set_inlet(const int *inlet, const double *uprof, const double *vprof, int nprof,
                         unsigned long long seed)
{
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    if (nprof < 0 || (nprof > 0 && (!uprof || !vprof))) return set_err(LES_ERR_ARG, "set_inlet: bad profiles");
    for (int q = 0; q < 4; q++) {
        int b = inlet ? inlet[q] : 0;
        if (b < 0 || b > c.g.numbl) return set_err(LES_ERR_ARG, "set_inlet: block %d out of range", b);
        c.inlet[q] = b;
    }
    cudaFree(c.d_uprof);
    cudaFree(c.d_vprof);
    c.d_uprof = c.d_vprof = nullptr;
    c.nprof = nprof;
    c.inlet_seed = seed;
    if (nprof > 0) {
        LES_CUDA(cudaMalloc(&c.d_uprof, sizeof(double) * nprof));
        LES_CUDA(cudaMalloc(&c.d_vprof, sizeof(double) * nprof));
        LES_CUDA(cudaMemcpy(c.d_uprof, uprof, sizeof(double) * nprof, cudaMemcpyDefault));
        LES_CUDA(cudaMemcpy(c.d_vprof, vprof, sizeof(double) * nprof, cudaMemcpyDefault));
    }
    return 0;
}

int lester_fixed_inlet(double *hu, double *hv, double *hw, double *u_int, double *v_int, double *w_int, double *u,
                       double *v, double *w, const double *p, double *sc1, double *rho, const double *gam,
                       const int *iseed, const double *y, const double *uprof, const double *vprof,
                       const double *wprof, const double *uuprof, const double *vvprof, const double *wwprof,
                       const double *umean, const double *vmean, const double *wmean, const double *uumean,
                       const double *vvmean, const double *wwmean, const int *step)
{
    (void)hu, (void)hv, (void)hw, (void)p, (void)gam, (void)y, (void)wprof, (void)uuprof, (void)vvprof;
    (void)wwprof, (void)umean, (void)vmean, (void)wmean, (void)uumean, (void)vvmean, (void)wwmean;
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    if (!step || !iseed) return set_err(LES_ERR_ARG, "fixed_inlet: NULL step / iseed");
    if (!has_inlet(c)) return 0;
    if (c.nprof <= 0 || !uprof || !vprof)
        return set_err(LES_ERR_ARG, "fixed_inlet: profiles and their length (lester_gpu_set_inlet) required");
    Staging st(&c, __func__);
    int r;
    const double *dp[2];
    if ((r = st.in(uprof, c.nprof, &dp[0])) || (r = st.in(vprof, c.nprof, &dp[1]))) return r;
    double *d[8];
    double *io3[8] = {u, v, w, sc1, rho, u_int, v_int, w_int};
    for (int q = 0; q < 8; q++)
        if ((r = st.io(io3[q], c.tot_sg3, &d[q]))) return r;
    if ((r = inlet_task(c, dp[0], dp[1], (unsigned long long)(unsigned)*iseed, *step, d[0], d[1], d[2], d[3], d[4],
                        d[5], d[6], d[7])))
        return r;
    return st.finish();
}

int lester_recycling(double *hu, double *hv, double *hw, double *u_int, double *v_int, double *w_int, double *u,
                     double *v, double *w, const double *p, double *sc1, double *rho, const double *gam, const int *iseed,
                     const double *y, const double *uprof, const double *vprof, const double *wprof,
                     const double *uuprof, const double *vvprof, const double *wwprof, double *umean, double *vmean,
                     double *wmean, double *uumean, double *vvmean, double *wwmean, const int *step,
                     const int *inblock)
{
    (void)hu, (void)hv, (void)hw, (void)p, (void)gam, (void)iseed, (void)y;
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    if (!step || !inblock) return set_err(LES_ERR_ARG, "recycling: NULL step / inblock");
    if (*inblock < 1 || *inblock > c.g.numbl) return set_err(LES_ERR_ARG, "recycling: inblock %d", *inblock);
    if (*inblock + 7 > c.g.numbl)
        return set_err(LES_ERR_ARG, "recycling: the chain %d..%d needs %d blocks", *inblock, *inblock + 7,
                       *inblock + 7);
    if (c.nprof <= 0) return set_err(LES_ERR_ARG, "recycling: profile length not set (lester_gpu_set_inlet)");
    Staging st(&c, __func__);
    int r;
    const double *pin[6] = {uprof, vprof, wprof, uuprof, vvprof, wwprof};
    const double *dpro[6];
    for (int q = 0; q < 6; q++)
        if ((r = st.in(pin[q], c.nprof, &dpro[q]))) return r;
    double *pio[6] = {umean, vmean, wmean, uumean, vvmean, wwmean};
    double *dm[6];
    for (int q = 0; q < 6; q++)
        if ((r = st.io(pio[q], c.nprof, &dm[q]))) return r;
    double *d3[8];
    double *io3[8] = {u, v, w, sc1, rho, u_int, v_int, w_int};
    for (int q = 0; q < 8; q++)
        if ((r = st.io(io3[q], c.tot_sg3, &d3[q]))) return r;
    std::vector<int> nijk(3 * c.g.numbl);
    long wl = 0;
    int njmax = 0;
    for (int b = 1; b <= c.g.numbl; b++) {
        for (int a = 0; a < 3; a++) nijk[3 * (b - 1) + a] = c.lv[1].n[b][a];
        wl = std::max(wl, 3L * (c.lv[1].n[b][1] + 1) * (c.lv[1].n[b][2] + 1));
        njmax = std::max(njmax, c.lv[1].n[b][1]);
    }
    int jmult = 0;
    if (*inblock == c.inlet[2]) jmult = 0;
    if (*inblock == c.inlet[1]) jmult = c.lv[1].n[*inblock][1] - 2;
    if (njmax + jmult > c.nprof) return set_err(LES_ERR_ARG, "recycling: profiles shorter than %d", njmax + jmult);
    double *work = nullptr;
    if (cudaMalloc(&work, sizeof(double) * wl) != cudaSuccess) {
        cudaGetLastError();
        return set_err(LES_ERR_NOMEM, "recycling: work");
    }
    RecycProf P;
    for (int q = 0; q < 3; q++) {
        P.mean[q] = dm[q];
        P.rms[q] = dm[3 + q];
        P.prof[q] = dpro[q];
        P.rprof[q] = dpro[3 + q];
    }
    launch_recycling(c.lv[1].d_blk, nijk.data(), c.g.numbl, *step, *inblock, jmult, c.c.rhohi, P, d3[0], d3[1],
                     d3[2], d3[3], d3[4], d3[5], d3[6], d3[7], work, c.stream);
    cudaError_t e = cudaStreamSynchronize(c.stream);
    cudaFree(work);
    if (e != cudaSuccess) return set_err(LES_ERR_CUDA, "recycling: %s", cudaGetErrorString(e));
    return st.finish();
}

int lester_gpu_set_stat_samples(int no_sam)
{
    LES_NEED_CTX();
    if (no_sam < 1) return set_err(LES_ERR_ARG, "statistics: no_sam must be >= 1");
    g_ctx->no_sam = no_sam;
    return 0;
}

int lester_statistics(const double *u, const double *v, const double *w, const double *p, const double *rho,
                      double *um, double *vm, double *wm, double *pm, double *rhom, double *ruv, double *rvw,
                      double *rwu, double *ruu, double *rvv, double *rww, double *rrh, const double *gam,
                      const double *gamsc1, const double *sc1, double *fm, double *rff, const double *sc1var,
                      const double *sc1dis, double *sc1varm, double *sc1dism, const double *temperature, double *t_m,
                      const double *dip, const double *djp, const double *rp, const double *dkp, const double *dkw,
                      const double *x, const double *y, const double *z, const int *step)
{
    (void)gamsc1, (void)sc1dis, (void)sc1dism, (void)temperature, (void)dip, (void)djp, (void)rp, (void)dkp;
    (void)dkw, (void)x, (void)y, (void)z, (void)step;
    LES_NEED_CTX();
    Ctx &c = *g_ctx;
    Staging st(&c, __func__);
    int r;
    const double *in[8] = {u, v, w, p, rho, sc1, sc1var, gam};
    const double *d[8];
    for (int q = 0; q < 8; q++)
        if ((r = st.in(in[q], c.tot_sg3, &d[q]))) return r;
    double *outs[16] = {um, vm, wm, pm, rhom, ruv, rvw, rwu, ruu, rvv, rww, rrh, fm, rff, sc1varm, t_m};
    StatOut O;
    long n2 = 0;
    for (int b = 1; b <= c.g.numbl; b++) n2 += (long)c.lv[1].n[b][0] * c.lv[1].n[b][1];
    for (int q = 0; q < 16; q++)
        if ((r = st.io(outs[q], n2, &O.f[q]))) return r;
    double *tmp = nullptr;
    if (cudaMalloc(&tmp, sizeof(double) * 3 * c.tot_sg3) != cudaSuccess) {
        cudaGetLastError();
        return set_err(LES_ERR_NOMEM, "statistics: centred velocities");
    }
    cudaMemsetAsync(tmp, 0, sizeof(double) * 3 * c.tot_sg3, c.stream);
    long maxpts = 0, maxij = 0;
    for (int b = 1; b <= c.g.numbl; b++) {
        const int *n = c.lv[1].n[b];
        maxpts = std::max(maxpts, (long)n[0] * n[1] * n[2]);
        maxij = std::max(maxij, (long)n[0] * n[1]);
    }
    launch_statistics(c.lv[1].d_blk, c.g.numbl, maxpts, maxij, c.no_sam, d[0], d[1], d[2], d[3], d[4], d[5], d[6],
                      d[7], tmp, tmp + c.tot_sg3, tmp + 2 * c.tot_sg3, O, c.stream);
    cudaError_t e = cudaStreamSynchronize(c.stream);
    cudaFree(tmp);
    if (e != cudaSuccess) return set_err(LES_ERR_CUDA, "statistics: %s", cudaGetErrorString(e));
    return st.finish();
}

} // extern "C"
