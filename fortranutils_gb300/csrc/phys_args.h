// phys_args.h -- argument bundles of the predictor and scalar kernels
// (passed by value; every pointer is a device pointer).
#pragma once

// metrics used by set_w_int / set_sc1 (their Fortran argument lists)
enum { MW_DIP, MW_DIU, MW_RDIV, MW_DJP, MW_DJV, MW_RDJU, MW_DIDJP, MW_RDIDJP, MW_HKIP, MW_HKJP,
       MW_HKIU, MW_HKJV, MW_RP, MW_RU, MW_N };

// set_u_int_block arguments in the roles set_uv_int gives them (for the v
// component the caller passes the swapped arrays, as code/step.F:319-326)
struct UIntArgs {
    const double *dip, *diu, *dix, *rdix, *djp, *dju, *djv, *djx, *rdjp, *rdju;
    const double *didjp, *didju, *rdidju, *hijp, *hiju, *hjiu, *hkiu, *hkju, *rp, *ru;
    const double *dkp, *dkw;
    const double *u, *v, *w, *p, *rho, *rhonp1, *gam;
    double *u_int, *hu;
    double *tw_s, *tw_n, *tw_l, *tw_r;
    const long *off_ki, *off_jk;  // per-block offsets of the (k,i) and (j,k) wall arrays
    long off2_lev1_base;          // 0: level-1 (i,j) arrays start with block 1
    // fast variant only: reciprocals of the divisor metrics (same layout)
    const double *r_dip, *r_diu, *r_dix, *r_djp, *r_dju, *r_djv, *r_djx, *r_rp, *r_dkp, *r_dkw;
    const double *fb;  // body force of this component per unit volume, or null
    const int *iststep;  // replayed graphs: the step counter on the device, or null
};

struct WIntArgs {
    const double *m[MW_N];
    const double *dkp, *dkw;
    const double *u, *v, *w, *p, *rho, *rhonp1, *gam;
    double *w_int, *hw;
    double *tw_sfk, *tw_nfk, *tw_wfk, *tw_efk;
    const long *off_ki, *off_jk;
    const double *r[MW_N];        // fast variant only: reciprocals of m[]
    const double *rdkp, *rdkw;
    const double *fb;             // body force of w per unit volume, or null
    const int *iststep;           // replayed graphs: the step counter on the device, or null
};

struct Sc1Args {
    const double *m[MW_N];
    const double *dkp, *dkw;
    const double *u, *v, *w, *rho, *gamsc1, *gamlam;
    double *sc1, *hsc1;
    const double *grad;  // interface gradients: per block 6 planes of gm*gm
    long gstride;
    int gm;
    const int *link;     // bl2bl, 0-based block numbers, 6 per block (-1 none)
    const double *r[MW_N];  // fast variant only: reciprocals of m[]
    const double *rdkp;
};

// grid barrier state of the persistent scalar sweep (zeroed before each
// launch): arrivals, the last completed barrier, and the timeout flag
struct WaveSync {
    unsigned count, gen;
    int err, pad;
};

// eddy viscosity and scalar variance, fast variant only: reciprocals of
// the divisor metrics and the filter width split as
// delta2d(i,j) * delta1d(k) = (dip*djp*rp)^0.33333333 * dkp^0.33333333
struct SgsFast {
    const double *r_dip, *r_djp, *r_rp, *r_dkp, *r_dkw, *delta2d, *delta1d;
};

// base, tangent and adjoint arrays of the linearised predictor inputs, in
// slot-field order: role-u, role-v, w, p, old h, body force, eddy
// viscosity (any may be null: zero)
struct PredRefs {
    const double *f[7];
};
struct PredBars {
    double *f[7];
};

// set_virt_bc arguments: the field, the wall array of the side being
// processed and the metrics the velocity branches read
struct VbcArgs {
    double *f, *vdd;
    const double *rho, *tw;
    const double *dju, *djx, *ru, *rv, *div_, *dix, *dip, *diu, *djp, *djv, *dkp, *dkw;
    const long *off_ki, *off_jk;
};
