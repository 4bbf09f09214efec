// k_graph.cu -- device-side control of the fast solve's cycle loop inside
// the whole-step graph (lester_step with ctrl.step_graph).
//
// The loop state d_loop (doubles):
//   0  ||b||^2 (compatible part), 1 relative residual, 2 previous one,
//   3  cycles run, 4 status, 6 the scalar sweep's barrier flag.
// Status: 0 cycling, 1 converged, 2 max_outer cycles reached, 3 a defect
// correction cycle failed to halve the residual (the host continues in
// flexible CG), 4 non-finite residual, 5 the flexible CG residual missed
// the tolerance once recomputed as b - A p (the host restarts the CG).
// Each kernel is one thread; every decision the host loop of
// fast_solve_run takes after a cycle is taken here in the same order.
#include <cuda_runtime.h>

#include "kernels.h"

namespace {

__global__ void k_loop_init(cudaGraphConditionalHandle h, const double *__restrict__ small,
                            double *__restrict__ loop, double rtol)
{
    const double r2 = small[0], b2 = small[1];
    const bool fin = isfinite(r2) && isfinite(b2);
    const double rel = b2 > 0 ? sqrt(r2 / b2) : 0.;
    const int go = fin && b2 > 0 && rel > rtol;
    loop[0] = b2;
    loop[1] = rel;
    loop[2] = rel;
    loop[3] = 0;
    loop[4] = !fin ? 4 : go ? 0 : 1;
    cudaGraphSetConditional(h, go);
}

__global__ void k_loop_step(cudaGraphConditionalHandle h, const double *__restrict__ small,
                            double *__restrict__ loop, double rtol, int maxit, int may_switch)
{
    const double prev = loop[1];
    const double rel = sqrt(small[0] / loop[0]);
    const int it = (int)loop[3] + 1;
    int st;
    if (!isfinite(rel)) st = 4;
    else if (may_switch && rel > rtol && rel > 0.5 * prev) st = 3;
    else if (rel <= rtol) st = 1;
    else if (it >= maxit) st = 2;
    else st = 0;
    loop[1] = rel;
    loop[2] = prev;
    loop[3] = it;
    loop[4] = st;
    cudaGraphSetConditional(h, st == 0);
}

// after the loop: the flexible CG's converged residual checked against the
// recomputed b - A p (confirm), then the gate of the rest of the step: run
// it when the solve converged or used its cycles, as the host path does
__global__ void k_loop_gate(cudaGraphConditionalHandle h, const double *__restrict__ small,
                            double *__restrict__ loop, double rtol, int confirm)
{
    int st = (int)loop[4];
    if (confirm && st == 1) {
        const double rel = sqrt(small[0] / loop[0]);
        loop[1] = rel;
        if (rel > rtol) st = 5;
        loop[4] = st;
    }
    cudaGraphSetConditional(h, st == 1 || st == 2);
}

__global__ void k_copy_flag(const int *__restrict__ src, double *__restrict__ dst) { *dst = (double)*src; }

// The fast solves' initial pressure in lester_step (ctrl.p_guess 1): when
// pp holds the pressure the previous step started its solve from, and that
// step was not the first (its p was a solution then),
// p <- 2 p - pp (linear extrapolation in time); pp <- the p found here
// either way.  The step number comes from istep_dev when given (a replayed
// graph) and saved holds the step pp was taken at.
__global__ void k_p_guess(double *__restrict__ p, double *__restrict__ pp, long n, int istep,
                          const int *__restrict__ istep_dev, const int *__restrict__ saved)
{
    const int st = istep_dev ? *istep_dev : istep;
    const bool extrap = *saved == st - 1 && st - 1 >= 2;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const double t = p[q];
        if (extrap) p[q] = 2.0 * t - pp[q];
        pp[q] = t;
    }
}

__global__ void k_p_guess_mark(int istep, const int *__restrict__ istep_dev, int *__restrict__ saved)
{
    *saved = istep_dev ? *istep_dev : istep;
}

} // namespace

namespace les {

void launch_loop_init(cudaGraphConditionalHandle h, const double *small, double *loop, double rtol,
                      cudaStream_t st)
{
    k_loop_init<<<1, 1, 0, st>>>(h, small, loop, rtol);
    count_launch(1);
}

void launch_loop_step(cudaGraphConditionalHandle h, const double *small, double *loop, double rtol, int maxit,
                      int may_switch, cudaStream_t st)
{
    k_loop_step<<<1, 1, 0, st>>>(h, small, loop, rtol, maxit, may_switch);
    count_launch(1);
}

void launch_loop_gate(cudaGraphConditionalHandle h, const double *small, double *loop, double rtol, int confirm,
                      cudaStream_t st)
{
    k_loop_gate<<<1, 1, 0, st>>>(h, small, loop, rtol, confirm);
    count_launch(1);
}

void launch_p_guess(double *p, double *pp, long n, int istep, const int *istep_dev, int *saved, cudaStream_t st)
{
    unsigned g = (unsigned)((n + 255) / 256);
    k_p_guess<<<g > 2432 ? 2432 : g, 256, 0, st>>>(p, pp, n, istep, istep_dev, saved);
    k_p_guess_mark<<<1, 1, 0, st>>>(istep, istep_dev, saved);
    count_launch(2);
}

void launch_copy_flag(const int *src, double *dst, cudaStream_t st)
{
    k_copy_flag<<<1, 1, 0, st>>>(src, dst);
    count_launch(1);
}

} // namespace les
