/*
 * orc_internal.h -- oracle private state.  TEST INFRASTRUCTURE ONLY.
 *
 * The context holds what the reference keeps in COMMON blocks:
 * cb.lgrid.inc (block sizes, links, offsets, multigrid dims),
 * cb.lcontrol.inc (cyclic tables, loop bounds, npts_all),
 * cb.comm.inc (face tables inikoff/inwoff/iniknum) and the SAVEd
 * smoother counter `jumble` (code/sporlx.F:58).
 */
#ifndef ORC_INTERNAL_H
#define ORC_INTERNAL_H
#include "lester_oracle.h"

/* 1-based Fortran element access on a 0-based C pointer */
#define A(p, idx) ((p)[(idx) - 1])
/* column-major 2-D (nip1, *) access, 1-based */
#define A2(p, i, j, n1) ((p)[((long)(i) - 1) + (long)(n1) * ((long)(j) - 1)])

/* cyclic(m, d) and cyclic1(m, d) of code/set_const.F:16-28, m = 1..2 */
extern const int orc_cyclic[2][4];
extern const int orc_cyclic1[2][4];
#define ORC_CYC(m, d) (orc_cyclic[(m) - 1][(d)])
#define ORC_CYC1(m, d) (orc_cyclic1[(m) - 1][(d)])

struct orc_ctx {
    int numbl, nummgl, maxmgl;
    int bl_nijkp1[ORC_MAXBL + 1][3];
    int bl_bc[ORC_MAXBL + 1][6];
    int bl2bl[ORC_MAXBL + 1][6];
    int bl2side[ORC_MAXBL + 1][6];
    int mg_nijkp1[ORC_MAXMGL + 1][ORC_MAXBL + 1][3];
    int mult[ORC_MAXMGL + 1][ORC_MAXBL + 1][3];
    long off3[ORC_MAXMGL + 1][ORC_MAXBL + 1];
    long off2[ORC_MAXMGL + 1][ORC_MAXBL + 1];
    long off1k[ORC_MAXMGL + 1][ORC_MAXBL + 1];
    long offxy[ORC_MAXMGL + 1][ORC_MAXBL + 1];
    long offz[ORC_MAXMGL + 1][ORC_MAXBL + 1];
    long offki[ORC_MAXMGL + 1][ORC_MAXBL + 1];
    long offjk[ORC_MAXMGL + 1][ORC_MAXBL + 1];
    long tot3, tot_sg3, tot2, tot1k, totxy, totz, tot_ki, tot_jk;
    long inikoff[ORC_MAXMGL + 1][ORC_MAXBL + 1][6][6];
    long inwoff[ORC_MAXMGL + 1][ORC_MAXBL + 1][6];
    int iniknum[ORC_MAXMGL + 1][ORC_MAXBL + 1][6][2];
    long inoffmax[ORC_MAXMGL + 1];
    long lwork;
    double *work;
    int nijkse[ORC_MAXMGL + 1][ORC_MAXBL + 1][6];
    double npts_all[ORC_MAXMGL + 1];
    int jumble;
    double rnorm[ORC_MAXMGL + 1], fnorm[ORC_MAXMGL + 1], enorm[ORC_MAXMGL + 1], vnorm[ORC_MAXMGL + 1];
    double tolc;
    /* conv_exitbc's SAVEd values (code/conv_exitbc.F:78): per-side outflow
       mass flux and rho-weighted area at step n, inflow and outflow sums */
    double exit_mflux_ttl[7], exit_arho_ttl[7], exit_mflux_in, exit_mflux_out;
    /* fixed_inlet: inlet block numbers (COMMON inlet1..inlet4), profiles */
    int inlet[4];
    double *uprof, *vprof;
    unsigned long long inlet_seed;
};

#endif
