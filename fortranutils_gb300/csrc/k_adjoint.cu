// k_adjoint.cu -- tangent-linear and adjoint kernels of the time step.
//
// The momentum predictor's per-point arithmetic (code/set_u_int_block.F,
// code/set_w_int_block.F, as k_phys.cu computes it) is restated here as a
// function template of the number type, with the inputs that are
// differentiated -- the velocities of its stencil, p, the previous explicit
// term h and the body force -- passed in a slot array, and evaluated with
// Dual<1> numbers: seeded by a tangent it gives the tangent-linear
// predictor (which the tests check against finite differences of the
// forward step); seeded by the unit vector of one slot it gives one entry
// of each point's Jacobian row, which the adjoint kernels scatter.  The eddy viscosity
// gam, the densities and the wall-stress running means are inputs that are
// not differentiated (their values come from the forward trajectory).
//
// The projection operators (sour_p, uvw_adv, extrap_p, p_ref_subtract, the
// face copies) are linear; their transposes are written out below.
#include "k_common.cuh"
#include "kernels.h"
#include "dual.cuh"

#define IDX2(b, i, j) ((b).off2 + ((i) - 1) + (long)(b).n[0] * ((j) - 1))

// slots of the u/v predictor inputs, in the roles set_uv_int gives them
enum { SU_P, SU_W, SU_E, SU_S, SU_N, SU_L, SU_R, SV_P, SV_N, SV_W, SV_NW, SW_P, SW_R, SW_W, SW_WR,
       SP_P, SP_W, SH_P, SF_P, SG_P, SG_W, SG_S, SG_SW, SG_N, SG_NW, SG_L, SG_WL, SG_R, SG_WR, NSU };
// slots of the w predictor inputs
enum { TU_P, TU_L, TU_E, TU_EL, TV_P, TV_L, TV_N, TV_NL, TW_P, TW_L, TW_R, TW_W, TW_E, TW_S, TW_N,
       TP_P, TP_L, TH_P, TF_P, TG_P, TG_L, TG_W, TG_WL, TG_E, TG_EL, TG_S, TG_SL, TG_N, TG_NL, NSW };

struct UPoint {
    long ijk, ijkw, ijke, ijks, ijkn, ijkl, ijkr, ijknw, ijkwr, ijksw, ijkwl;
    long ij, ijw, ijn, ijs, ijnw;
    int i, j, k;  // role coordinates
};

// role geometry of point (ir, jr, k) of the u (iva 1) or v (iva 2) predictor;
// false if the point is not updated (first interior plane of a
// non-periodic side, set_u_int_block.F istart)
__device__ __forceinline__ bool upoint(const BlkDev &b, int iva, long ijk, int ir, int jr, int k, UPoint &P)
{
    int i = iva == 1 ? ir : jr, j = iva == 1 ? jr : ir;
    long io = iva == 1 ? 1 : b.n[0], jo = iva == 1 ? b.n[0] : 1, ko = (long)b.n[0] * b.n[1];
    int s0 = b.bc[iva == 1 ? 0 : 2];
    int istart = (s0 != LES_BCT_PERIODIC_D && s0 != LES_BCT_INTERFACE_D) ? 3 : 2;
    if (i < istart) return false;
    P.i = i;
    P.j = j;
    P.k = k;
    P.ijk = ijk;
    P.ijkw = ijk - io;
    P.ijke = ijk + io;
    P.ijks = ijk - jo;
    P.ijkn = ijk + jo;
    P.ijkl = ijk - ko;
    P.ijkr = ijk + ko;
    P.ijknw = P.ijkn - io;
    P.ijkwr = P.ijkw + ko;
    P.ijksw = P.ijks - io;
    P.ijkwl = P.ijkw - ko;
    P.ij = b.off2 + io * (i - 1) + jo * (j - 1);
    P.ijw = P.ij - io;
    P.ijs = P.ij - jo;
    P.ijn = P.ij + jo;
    P.ijnw = P.ijw + jo;
    return true;
}

// set_u_int_block.F:103-462 for one point; in[] holds the slot values
template <typename R>
__device__ void upred_cell(const BlkDev &b, int bi, int iva, const UPoint &P, const UIntArgs &A_,
                           double dtime, double visc, double ylaminar, double kappa, double cwfun,
                           const R *in, R &u_int, R &hout)
{
    const int i = P.i, j = P.j, k = P.k;
    const long ijk = P.ijk, ijkw = P.ijkw, ijks = P.ijks, ijkn = P.ijkn, ijkl = P.ijkl, ijkr = P.ijkr;
    const long ijknw = P.ijknw, ijkwr = P.ijkwr;
    const long ij = P.ij, ijw = P.ijw, ijn = P.ijn, ijs = P.ijs, ijnw = P.ijnw;
    const long io = P.ijke - ijk, jo = ijkn - ijk, ko = ijkr - ijk;
    const long ijksw = P.ijksw, ijkwl = P.ijkwl;
    const int nkp1 = b.n[2], nj = (iva == 1 ? b.n[1] : b.n[0]) - 1, nk = nkp1 - 1;
    const bool wallsf = b.bc[iva == 1 ? 2 : 0] == LES_BCT_WALL_D;
    const bool wallnf = b.bc[iva == 1 ? 3 : 1] == LES_BCT_WALL_D;
    const bool walllf = b.bc[4] == LES_BCT_WALL_D, wallrf = b.bc[5] == LES_BCT_WALL_D;
    const double *rho = A_.rho;
    const double *dkp = A_.dkp + b.off1k, *dkw = A_.dkw + b.off1k;
    const double di = A_.diu[ij], dj = A_.dju[ij];
    const double rdkp = A_.rp[ij] * dkp[k - 1];
    const double rdku = A_.ru[ij] * dkp[k - 1];
    const R uP = in[SU_P], uW = in[SU_W], uE = in[SU_E], uS = in[SU_S], uN = in[SU_N], uL = in[SU_L],
            uR = in[SU_R];
    const R vP = in[SV_P], vN = in[SV_N], vW = in[SV_W], vNW = in[SV_NW];
    const R wP = in[SW_P], wR = in[SW_R], wW = in[SW_W], wWR = in[SW_WR];
    R va = 0.25 * (vP + vN + vW + vNW);
    R wa = 0.25 * (wP + wR + wW + wWR);
    double rhoa = 0.5 * (rho[ijkw] + rho[ijk]);
    // the eddy viscosity is an input slot (differentiated through the
    // subgrid model); the densities are not
    const R gP = in[SG_P], gW = in[SG_W], gS = in[SG_S], gSW = in[SG_SW], gN = in[SG_N], gNW = in[SG_NW],
            gL = in[SG_L], gWL = in[SG_WL], gR = in[SG_R], gWR = in[SG_WR];
    R gama = 0.5 * (gW + gP);
    double rhowf = rho[ijkw], rhoef = rho[ijk];
    double rhosf = 0.25 * (rho[ijk] + rho[ijkw] + rho[ijks] + rho[ijksw]);
    double rhonf = 0.25 * (rho[ijk] + rho[ijkw] + rho[ijkn] + rho[ijknw]);
    double rholf = 0.25 * (rho[ijk] + rho[ijkw] + rho[ijkl] + rho[ijkwl]);
    double rhorf = 0.25 * (rho[ijk] + rho[ijkw] + rho[ijkr] + rho[ijkwr]);
    double rhou = 0.5 * (rho[ijk] + rho[ijkw]);
    double rhonp1u = 0.5 * (A_.rhonp1[ijk] + A_.rhonp1[ijkw]);
    R gamwf = visc + gW * rhowf;
    R gamef = visc + gP * rhoef;
    R gamsf = visc + .25 * (gP + gW + gS + gSW) * rhosf;
    R gamnf = visc + .25 * (gP + gW + gN + gNW) * rhonf;
    R gamlf = visc + .25 * (gP + gW + gL + gWL) * rholf;
    R gamrf = visc + .25 * (gP + gW + gR + gWR) * rhorf;
    double areawf = A_.rdjp[ijw] * dkp[k - 1];
    double areaef = A_.rdjp[ij] * dkp[k - 1];
    double areasf = A_.rdix[ij] * dkp[k - 1];
    double areanf = A_.rdix[ijn] * dkp[k - 1];
    double areak = A_.didju[ij];
    double vol = A_.rdidju[ij] * dkp[k - 1];
    R uwf = 0.5 * (uP + uW);
    R uef = 0.5 * (uP + uE);
    R vsf = 0.5 * (vP + vW);
    R vnf = 0.5 * (vN + vNW);
    R wlf = 0.5 * (wP + wW);
    R wrf = 0.5 * (wR + wWR);
    R gwf = uwf * uwf * rhowf * areawf;
    R gef = uef * uef * rhoef * areaef;
    R gsf = 0.5 * (uP + uS) * vsf * rhosf * areasf;
    R gnf = 0.5 * (uP + uN) * vnf * rhonf * areanf;
    R glf = 0.5 * (uP + uL) * wlf * rholf * areak;
    R grf = 0.5 * (uP + uR) * wrf * rhorf * areak;
    R conf = -(gef - gwf) - (gnf - gsf) - (grf - glf);
    R cc1 = A_.hjiu[ij] * rhoa * (va * va) * vol;
    R cc2 = A_.hkiu[ij] * rhoa * (wa * wa) * vol;
    R cc3 = -A_.hiju[ij] * rhoa * va * uP * vol;
    R conc = cc1 + cc2 + cc3;
    R galwf = gamwf * areawf / A_.dip[ijw];
    R galef = gamef * areaef / A_.dip[ij];
    R galsf = gamsf * areasf / A_.djx[ij];
    R galnf = gamnf * areanf / A_.djx[ijn];
    R gallf = gamlf * areak / (A_.rp[ij] * dkw[k - 1]);
    R galrf = gamrf * areak / (A_.rp[ij] * dkw[k]);
    R vwf = 0.5 * (vW + vNW);
    R vef = 0.5 * (vP + vN);
    R twf = galwf * 2.0 * (uP - uW);
    R tef = galef * 2.0 * (uE - uP);
    R tsf = galsf * A_.dix[ij] * (uP / A_.diu[ij] - uS / A_.diu[ijs]);
    R tnf = galnf * A_.dix[ijn] * (uN / A_.diu[ijn] - uP / A_.diu[ij]);
    R tlf = gallf * (uP - uL);
    R trf = galrf * (uR - uP);
    R cwf = 2.0 * gamwf * areawf * vwf * A_.hijp[ijw];
    R cef = 2.0 * gamef * areaef * vef * A_.hijp[ij];
    R csf = gamsf * areasf * A_.djx[ij] * (vP / A_.djv[ij] - vW / A_.djv[ijw]) / A_.dix[ij];
    R cnf = gamnf * areanf * A_.djx[ijn] * (vN / A_.djv[ijn] - vNW / A_.djv[ijnw]) / A_.dix[ijn];
    R clf = gamlf * areak * A_.ru[ij] * (wP / A_.rp[ij] - wW / A_.rp[ijw]) / A_.diu[ij];
    R crf = gamrf * areak * A_.ru[ij] * (wR / A_.rp[ij] - wWR / A_.rp[ijw]) / A_.diu[ij];
    R tiiwf = twf + cwf, tiief = tef + cef, tjisf = tsf + csf, tjinf = tnf + cnf;
    R tkilf = tlf + clf, tkirf = trf + crf;
    R dc1 = -2.0 * gama * vol * A_.hjiu[ij] * ((vnf - vsf) / A_.dju[ij] + uP * A_.hjiu[ij]);
    R dc2 = -2.0 * gama * vol * A_.hkiu[ij] * (uP * A_.hkiu[ij] + va * A_.hkju[ij] + (wrf - wlf) / rdkp);
    R udisf = 0.5 * (uP + uS) / A_.dix[ij];
    R udinf = 0.5 * (uP + uN) / A_.dix[ijn];
    R vdjwf = 0.5 * (vW + vNW) / A_.djp[ijw];
    R vdjef = 0.5 * (vP + vN) / A_.djp[ij];
    R dc3 = gama * vol * A_.hiju[ij] * (di * (udinf - udisf) / dj + dj * (vdjef - vdjwf) / di);
    R diffc = dc1 + dc2 + dc3;
    // wall stress (set_u_int_block.F:353-439) with the running means of the
    // forward state; tw is linear in the point's velocity in both branches
    long kio = (iva == 1 ? A_.off_ki : A_.off_jk)[bi];
    long ki = (k - 1) + (long)nkp1 * (i - 1);
    long ijl = (b.off2 - A_.off2_lev1_base) + (ij - b.off2);
    auto wall = [&](const double *twa, long at, double rf, double dist) -> R {
        double tw_mean = fabs(twa[at]);
        double ut_mean = sqrt(tw_mean / rf);
        double yplus_mean = dist * ut_mean * rf / visc;
        if (yplus_mean > ylaminar) {
            double uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
            return uP * tw_mean / uloglaw;
        }
        return visc * uP / dist;
    };
    if (wallsf && j == 2) tjisf = areasf * wall(A_.tw_s + kio, ki, rhosf, 0.5 * A_.dju[ij]);
    if (wallnf && j == nj) tjinf = -areanf * wall(A_.tw_n + kio, ki, rhonf, 0.5 * A_.dju[ij]);
    if (walllf && k == 2) tkilf = areak * wall(A_.tw_l, ijl, rholf, 0.5 * rdku);
    if (wallrf && k == nk) tkirf = -areak * wall(A_.tw_r, ijl, rhorf, 0.5 * rdku);
    R h = conf + conc + diffc + tiief - tiiwf + tjinf - tjisf + tkirf - tkilf;
    h = h + in[SF_P] * vol;
    u_int = uP * (rhou / rhonp1u) +
            dtime / (rhonp1u * vol) * (1.5 * h - 0.5 * in[SH_P] + 0.5 * (in[SP_P] - in[SP_W]) * vol / di);
    hout = h;
}

// the absolute positions of the u/v predictor slots
__device__ __forceinline__ void uslots(const UPoint &P, long *at, int *fld)
{
    // fld: 0 role-u, 1 role-v, 2 w, 3 p, 4 h, 5 body force, 6 eddy viscosity
    const long a[NSU] = {P.ijk,  P.ijkw, P.ijke, P.ijks, P.ijkn, P.ijkl,  P.ijkr, P.ijk,  P.ijkn, P.ijkw,
                         P.ijknw, P.ijk, P.ijkr, P.ijkw, P.ijkwr, P.ijk,  P.ijkw, P.ijk,  P.ijk,  P.ijk,
                         P.ijkw, P.ijks, P.ijksw, P.ijkn, P.ijknw, P.ijkl, P.ijkwl, P.ijkr, P.ijkwr};
    const int f[NSU] = {0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 4, 5, 6, 6, 6, 6, 6, 6, 6, 6, 6, 6};
#pragma unroll
    for (int q = 0; q < NSU; q++) {
        at[q] = a[q];
        fld[q] = f[q];
    }
}

// ---------------------------------------------------------------- w point
struct WPoint {
    long ijk, ijkw, ijke, ijks, ijkn, ijkl, ijkr, ijkwl, ijksl, ijkel, ijknl;
    int i, j, k;
};

// set_w_int_block.F:95-458 for one point
template <typename R>
__device__ void wpred_cell(const BlkDev &b, int bi, const WPoint &P, const WIntArgs &A_, double dtime,
                           double visc, double ylaminar, double kappa, double cwfun, const R *in,
                           R &w_int, R &hout)
{
    const int i = P.i, j = P.j, k = P.k;
    const long ijk = P.ijk, ijkw = P.ijkw, ijke = P.ijke, ijks = P.ijks, ijkn = P.ijkn, ijkl = P.ijkl;
    const long ijkwl = P.ijkwl, ijksl = P.ijksl, ijkel = P.ijkel, ijknl = P.ijknl;
    const int nkp1 = b.n[2], ni = b.n[0] - 1, nj = b.n[1] - 1;
    const double *rho = A_.rho;
    const double *dkp = A_.dkp + b.off1k, *dkw = A_.dkw + b.off1k;
    const double *const *M = A_.m;
#define G(a, ii, jj) M[a][IDX2(b, ii, jj)]
    double radp = G(MW_RP, i, j), radw = G(MW_RP, i - 1, j), rade = G(MW_RP, i + 1, j);
    double rads = G(MW_RP, i, j - 1), radn = G(MW_RP, i, j + 1);
    double rhowf = 0.25 * (rho[ijk] + rho[ijkl] + rho[ijkw] + rho[ijkwl]);
    double rhoef = 0.25 * (rho[ijk] + rho[ijkl] + rho[ijke] + rho[ijkel]);
    double rhosf = 0.25 * (rho[ijk] + rho[ijkl] + rho[ijks] + rho[ijksl]);
    double rhonf = 0.25 * (rho[ijk] + rho[ijkl] + rho[ijkn] + rho[ijknl]);
    double rholf = rho[ijkl], rhorf = rho[ijk];
    double rhow = 0.5 * (rho[ijk] + rho[ijkl]);
    double rhonp1w = 0.5 * (A_.rhonp1[ijk] + A_.rhonp1[ijkl]);
    const R gP = in[TG_P], gL = in[TG_L], gW = in[TG_W], gWL = in[TG_WL], gE = in[TG_E], gEL = in[TG_EL],
            gS = in[TG_S], gSL = in[TG_SL], gN = in[TG_N], gNL = in[TG_NL];
    R gamwf = visc + .25 * (gP + gL + gW + gWL) * rhowf;
    R gamef = visc + .25 * (gP + gL + gE + gEL) * rhoef;
    R gamsf = visc + .25 * (gP + gL + gS + gSL) * rhosf;
    R gamnf = visc + .25 * (gP + gL + gN + gNL) * rhonf;
    R gamlf = visc + gL * rholf;
    R gamrf = visc + gP * rhorf;
    double areawf = G(MW_RDJU, i, j) * dkw[k - 1];
    double areaef = G(MW_RDJU, i + 1, j) * dkw[k - 1];
    double areasf = G(MW_RDIV, i, j) * dkw[k - 1];
    double areanf = G(MW_RDIV, i, j + 1) * dkw[k - 1];
    double areak = G(MW_DIDJP, i, j);
    double vol = G(MW_RDIDJP, i, j) * dkw[k - 1];
    const R uP = in[TU_P], uL = in[TU_L], uE = in[TU_E], uEL = in[TU_EL];
    const R vP = in[TV_P], vL = in[TV_L], vN = in[TV_N], vNL = in[TV_NL];
    const R wP = in[TW_P], wL = in[TW_L], wR = in[TW_R], wW = in[TW_W], wE = in[TW_E], wS = in[TW_S],
            wN = in[TW_N];
    R uwf = 0.5 * (uP + uL);
    R uef = 0.5 * (uE + uEL);
    R vsf = 0.5 * (vP + vL);
    R vnf = 0.5 * (vN + vNL);
    R wlf = 0.5 * (wP + wL);
    R wrf = 0.5 * (wR + wP);
    R gwf = 0.5 * (wP + wW) * uwf * rhowf * areawf;
    R gef = 0.5 * (wP + wE) * uef * rhoef * areaef;
    R gsf = 0.5 * (wP + wS) * vsf * rhosf * areasf;
    R gnf = 0.5 * (wP + wN) * vnf * rhonf * areanf;
    R glf = wlf * wlf * rholf * areak;
    R grf = wrf * wrf * rhorf * areak;
    R conf = -(gef - gwf) - (gnf - gsf) - (grf - glf);
    R u_wc = 0.25 * (uP + uE + uL + uEL);
    R v_wc = 0.25 * (vP + vN + vL + vNL);
    R conc = -vol * rhow * (wP * (u_wc * G(MW_HKIP, i, j) + v_wc * G(MW_HKJP, i, j)));
    R galwf = gamwf * areawf / G(MW_DIU, i, j);
    R galef = gamef * areaef / G(MW_DIU, i + 1, j);
    R galsf = gamsf * areasf / G(MW_DJV, i, j);
    R galnf = gamnf * areanf / G(MW_DJV, i, j + 1);
    R gallf = gamlf * areak / (radp * dkp[k - 2]);
    R galrf = gamrf * areak / (radp * dkp[k - 1]);
    double radwf = 0.5 * (radp + radw), radef = 0.5 * (radp + rade);
    double radsf = 0.5 * (radp + rads), radnf = 0.5 * (radp + radn);
    R ulf = 0.5 * (uL + uEL), urf = 0.5 * (uP + uE);
    R vlf = 0.5 * (vL + vNL), vrf = 0.5 * (vP + vN);
    R wwf = 0.5 * (wP + wW), wef = 0.5 * (wP + wE);
    R wsf = 0.5 * (wP + wS), wnf = 0.5 * (wP + wN);
    R twf = galwf * radwf * (wP / radp - wW / radw);
    R tef = galef * radef * (wE / rade - wP / radp);
    R tsf = galsf * (wP - wS);
    R tnf = galnf * (wN - wP);
    R tlf = 2.0 * gallf * (wP - wL);
    R trf = 2.0 * galrf * (wR - wP);
    R cwf = gamwf * areawf * ((uP - uL) / dkw[k - 1] / radwf - wwf * G(MW_HKIU, i, j));
    R cef = gamef * areaef * ((uE - uEL) / dkw[k - 1] / radef - wef * G(MW_HKIU, i + 1, j));
    R csf = (j == 2) ? dconst_like(wP, 0.0)
                     : gamsf * areasf * ((vP - vL) / dkw[k - 1] / radsf - wsf * G(MW_HKJV, i, j));
    R cnf = gamnf * areanf * ((vN - vNL) / dkw[k - 1] / radnf - wnf * G(MW_HKJV, i, j + 1));
    R clf = 2.0 * gamlf * areak * (ulf * G(MW_HKIP, i, j) + vlf * G(MW_HKJP, i, j));
    R crf = 2.0 * gamrf * areak * (urf * G(MW_HKIP, i, j) + vrf * G(MW_HKJP, i, j));
    R dwdy = (wnf - wsf) / G(MW_DJP, i, j);
    R dvdz = (vrf - vlf) / (radp * dkw[k - 1]);
    R dwdx = (wef - wwf) / G(MW_DIP, i, j);
    R dudz = (urf - ulf) / (radp * dkw[k - 1]);
    R diffc1 = G(MW_HKIP, i, j) * (dwdx + dudz - wP * G(MW_HKIP, i, j)) * vol * gamrf;
    R diffc2 = G(MW_HKJP, i, j) * (dwdy + dvdz - wP * G(MW_HKJP, i, j)) * vol * gamrf;
    R diffc = diffc1 + diffc2;
    R tikwf = twf + cwf, tikef = tef + cef, tjksf = tsf + csf, tjknf = tnf + cnf;
    R tkklf = tlf + clf, tkkrf = trf + crf;
    const double w_wall = 0.0;
    long kj = A_.off_jk[bi] + (k - 1) + (long)nkp1 * (j - 1);
    long kii = A_.off_ki[bi] + (k - 1) + (long)nkp1 * (i - 1);
    auto wall = [&](const double *twa, long at, double rf, double dist) -> R {
        double tw_mean = fabs(twa[at]);
        double ut_mean = sqrt(tw_mean / rf);
        double yplus_mean = dist * ut_mean * rf / visc;
        if (yplus_mean > ylaminar) {
            double uloglaw = ut_mean / kappa * (log(yplus_mean) + cwfun);
            return wP * tw_mean / uloglaw;
        }
        return visc * (wP - w_wall) / dist;
    };
    if (b.bc[0] == LES_BCT_WALL_D && i == 2)
        tikwf = areawf * (wall(A_.tw_wfk, kj, rhowf, 0.5 * G(MW_DIP, i, j)) - w_wall / 0.005 * visc);
    if (b.bc[1] == LES_BCT_WALL_D && i == ni)
        tikef = -areaef * (wall(A_.tw_efk, kj, rhoef, 0.5 * G(MW_DIP, i, j)) + w_wall / 0.015 * visc);
    if (b.bc[2] == LES_BCT_WALL_D && j == 2)
        tjksf = areasf * (wall(A_.tw_sfk, kii, rhosf, 0.5 * G(MW_DJP, i, j)) - w_wall / 0.005 * visc);
    if (b.bc[3] == LES_BCT_WALL_D && j == nj)
        tjknf = -areanf * (wall(A_.tw_nfk, kii, rhonf, 0.5 * G(MW_DJP, i, j)) + w_wall / 0.015 * visc);
    R difff = tikef - tikwf + tjknf - tjksf + tkkrf - tkklf;
    R h = conf + conc + difff + diffc;
    h = h + in[TF_P] * vol;
    w_int = wP * (rhow / rhonp1w) +
            dtime / (vol * rhonp1w) * (1.5 * h - 0.5 * in[TH_P] + 0.5 * areak * (in[TP_P] - in[TP_L]));
    hout = h;
#undef G
}

// ------------------------------------------------------------- w slots
__device__ __forceinline__ void wslots(const WPoint &P, long *at, int *fld)
{
    // fld: 0 u, 1 v, 2 w, 3 p, 4 h, 5 body force
    const long a[NSW] = {P.ijk,  P.ijkl,  P.ijke, P.ijkel, P.ijk,  P.ijkl, P.ijkn, P.ijknl, P.ijk,  P.ijkl,
                         P.ijkr, P.ijkw,  P.ijke, P.ijks,  P.ijkn, P.ijk,  P.ijkl, P.ijk,   P.ijk,  P.ijk,
                         P.ijkl, P.ijkw, P.ijkwl, P.ijke, P.ijkel, P.ijks, P.ijksl, P.ijkn, P.ijknl};
    const int f[NSW] = {0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 3, 3, 4, 5, 6, 6, 6, 6, 6, 6, 6, 6, 6, 6};
#pragma unroll
    for (int q = 0; q < NSW; q++) {
        at[q] = a[q];
        fld[q] = f[q];
    }
}

__device__ __forceinline__ bool wpoint(const BlkDev &b, long ijk, int i, int j, int k, WPoint &P)
{
    int kstart = (b.bc[4] != LES_BCT_PERIODIC_D && b.bc[4] != LES_BCT_INTERFACE_D) ? 3 : 2;
    if (k < kstart) return false;
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    P.i = i;
    P.j = j;
    P.k = k;
    P.ijk = ijk;
    P.ijkw = ijk - 1;
    P.ijke = ijk + 1;
    P.ijks = ijk - jo;
    P.ijkn = ijk + jo;
    P.ijkl = ijk - ko;
    P.ijkr = ijk + ko;
    P.ijkwl = P.ijkw - ko;
    P.ijksl = P.ijks - ko;
    P.ijkel = P.ijke - ko;
    P.ijknl = P.ijkn - ko;
    return true;
}

// ------------------------------------------------- linearised predictors
// mode 0: tangent-linear -- inputs carry the tangents tan.f[], outputs are
//         written to out_u (the point's u_int tangent) and out_h.
// mode 1: adjoint pass for input slot q0 -- the seed is the unit vector of
//         slot q0; lam_u (adjoint of u_int) and lam_h (adjoint of the new h)
//         times the two derivatives are added to bar.f[fld(q0)] at that
//         slot's point.
// mode 2: forward value (tangents ignored) into out_u, out_h.
template <int NS, typename Pt, typename Args, typename Cell, typename Slots>
__device__ __forceinline__ void lin_point(int mode, int q0, const Pt &P, const Args &A_,
                                          const PredRefs &base, const PredRefs &tan,
                                          const PredBars &bar, const double *lam_u,
                                          const double *lam_h, double *out_u, double *out_h,
                                          Cell cell, Slots slots)
{
    long at[NS];
    int fld[NS];
    slots(P, at, fld);
    Dual<1> in[NS];
#pragma unroll
    for (int q = 0; q < NS; q++) {
        const double *bf = base.f[fld[q]];
        in[q].v = bf ? bf[at[q]] : 0.;
        if (mode == 0) {
            const double *tf = tan.f[fld[q]];
            in[q].d[0] = tf ? tf[at[q]] : 0.;
        } else {
            in[q].d[0] = (mode == 1 && q == q0) ? 1. : 0.;
        }
    }
    Dual<1> uo, ho;
    cell(in, uo, ho);
    if (mode == 0) {
        out_u[P.ijk] = uo.d[0];
        out_h[P.ijk] = ho.d[0];
    } else if (mode == 2) {
        out_u[P.ijk] = uo.v;
        out_h[P.ijk] = ho.v;
    } else {
        double c = lam_u[P.ijk] * uo.d[0] + lam_h[P.ijk] * ho.d[0];
        double *bf = bar.f[fld[q0]];
        if (bf && c != 0.) atomicAdd(bf + at[q0], c);
    }
}

__global__ void __launch_bounds__(128) k_upred_lin(const BlkDev *__restrict__ blk, int iva, int mode,
                                                   int q0, UIntArgs A_, PredRefs base, PredRefs tan,
                                                   PredBars bar, const double *lam_u,
                                                   const double *lam_h, double *out_u, double *out_h,
                                                   double dtime, double visc, double ylaminar,
                                                   double kappa, double cwfun)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int ir, jr, k;
    long ijk = decode_interior(b, q, ir, jr, k);
    UPoint P;
    if (!upoint(b, iva, ijk, ir, jr, k, P)) return;
    const int bi = blockIdx.y;
    lin_point<NSU>(mode, q0, P, A_, base, tan, bar, lam_u, lam_h, out_u, out_h,
                   [&](const Dual<1> *in, Dual<1> &uo, Dual<1> &ho) {
                       upred_cell(b, bi, iva, P, A_, dtime, visc, ylaminar, kappa, cwfun, in, uo, ho);
                   },
                   [](const UPoint &Pp, long *at, int *fld) { uslots(Pp, at, fld); });
}

__global__ void __launch_bounds__(128) k_wpred_lin(const BlkDev *__restrict__ blk, int mode, int q0,
                                                   WIntArgs A_, PredRefs base, PredRefs tan,
                                                   PredBars bar, const double *lam_u,
                                                   const double *lam_h, double *out_u, double *out_h,
                                                   double dtime, double visc, double ylaminar,
                                                   double kappa, double cwfun)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long ijk = decode_interior(b, q, i, j, k);
    WPoint P;
    if (!wpoint(b, ijk, i, j, k, P)) return;
    const int bi = blockIdx.y;
    lin_point<NSW>(mode, q0, P, A_, base, tan, bar, lam_u, lam_h, out_u, out_h,
                   [&](const Dual<1> *in, Dual<1> &uo, Dual<1> &ho) {
                       wpred_cell(b, bi, P, A_, dtime, visc, ylaminar, kappa, cwfun, in, uo, ho);
                   },
                   [](const WPoint &Pp, long *at, int *fld) { wslots(Pp, at, fld); });
}

// the new h of a point is the adjoint's output, consumed before the passes
// (its adjoint then only holds the derivative with respect to the old h)
__global__ void k_take(const BlkDev *__restrict__ blk, int iva_or_w, const double *__restrict__ src,
                       double *__restrict__ dst, double *__restrict__ zero_src)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long ijk = decode_interior(b, q, i, j, k);
    // only the points the predictor writes
    int c = iva_or_w == 1 ? i : iva_or_w == 2 ? j : k;
    int side = iva_or_w == 1 ? 0 : iva_or_w == 2 ? 2 : 4;
    int start = (b.bc[side] != LES_BCT_PERIODIC_D && b.bc[side] != LES_BCT_INTERFACE_D) ? 3 : 2;
    if (c < start) return;
    dst[ijk] = src[ijk];
    if (zero_src) zero_src[ijk] = 0.;
}

// ------------------------------------------------- linearised Smagorinsky
// subgrid_smagorinsky.F:85-222 (as k_sgs.cu computes it off polar grids) for
// one interior point: gam from 30 velocity slots (fields 0-2: u, v, w).
// The damping is a constant: set_virt_bc resets it to 1 on each of the
// step's three calls (set_virt_bc.F:72-74) and the w call's wall planes keep
// the larger of 1 and the van Driest value, so the step's gam sees 1.
enum { GU_P, GU_E, GU_S, GU_SE, GU_N, GU_NE, GU_L, GU_EL, GU_R, GU_ER,
       GV_P, GV_N, GV_W, GV_NW, GV_E, GV_NE, GV_L, GV_NL, GV_R, GV_NR,
       GW_P, GW_R, GW_W, GW_WR, GW_E, GW_ER, GW_S, GW_SR, GW_N, GW_NR, NSG };

template <typename R>
__device__ R smag_cell(const R *in, double di, double dj, double dk, double hijp, double hjip, double csles,
                       double vdd)
{
    R up = 0.5 * (in[GU_P] + in[GU_E]);
    R vp = 0.5 * (in[GV_P] + in[GV_N]);
    R vwf = 0.25 * (in[GV_P] + in[GV_N] + in[GV_W] + in[GV_NW]);
    R vef = 0.25 * (in[GV_P] + in[GV_N] + in[GV_E] + in[GV_NE]);
    R usf = 0.25 * (in[GU_P] + in[GU_E] + in[GU_S] + in[GU_SE]);
    R unf = 0.25 * (in[GU_P] + in[GU_E] + in[GU_N] + in[GU_NE]);
    R ulf = 0.25 * (in[GU_P] + in[GU_E] + in[GU_L] + in[GU_EL]);
    R urf = 0.25 * (in[GU_P] + in[GU_E] + in[GU_R] + in[GU_ER]);
    R vlf = 0.25 * (in[GV_P] + in[GV_N] + in[GV_L] + in[GV_NL]);
    R vrf = 0.25 * (in[GV_P] + in[GV_N] + in[GV_R] + in[GV_NR]);
    R dudi = (in[GU_E] - in[GU_P]) / di + vp * hijp;
    R dvdi = (vef - vwf) / di - up * hijp;
    R dudj = (unf - usf) / dj - vp * hjip;
    R dvdj = (in[GV_N] - in[GV_P]) / dj + up * hjip;
    R wwf = 0.25 * (in[GW_P] + in[GW_R] + in[GW_W] + in[GW_WR]);
    R wef = 0.25 * (in[GW_P] + in[GW_R] + in[GW_E] + in[GW_ER]);
    R wsf = 0.25 * (in[GW_P] + in[GW_R] + in[GW_S] + in[GW_SR]);
    R wnf = 0.25 * (in[GW_P] + in[GW_R] + in[GW_N] + in[GW_NR]);
    R dwdi = (wef - wwf) / di;
    R dwdj = (wnf - wsf) / dj;
    R dudk = (urf - ulf) / dk;
    R dvdk = (vrf - vlf) / dk;
    R dwdk = (in[GW_R] - in[GW_P]) / dk;
    R sijsij = dvdj * dvdj + dwdk * dwdk + dudi * dudi +
               0.5 * ((dudj + dvdi) * (dudj + dvdi) + (dvdk + dwdj) * (dvdk + dwdj) + (dudk + dwdi) * (dudk + dwdi));
    const double delta_xyz = pow(di * dj * dk, .33333333);
    const double evisc = csles * delta_xyz * vdd;
    return evisc * evisc * sqrt(2.0 * sijsij);
}

// mode 0: gam tangent from the velocity tangents into out; mode 1: pass for
// slot q0, lam (adjoint of gam) times the derivative added to the slot's
// velocity adjoint
__global__ void __launch_bounds__(128) k_sgs_lin(const BlkDev *__restrict__ blk, int mode, int q0, PredRefs base,
                                                 PredRefs tan, PredBars bar, const double *__restrict__ lam,
                                                 double *__restrict__ out, const double *__restrict__ dip,
                                                 const double *__restrict__ djp, const double *__restrict__ dkp,
                                                 const double *__restrict__ hijp, const double *__restrict__ hjip,
                                                 const double *__restrict__ vdd, double csles)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    const long ijk = decode_interior(b, q, i, j, k);
    const long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    const long at[NSG] = {ijk, ijk + 1, ijk - jo, ijk - jo + 1, ijk + jo, ijk + jo + 1, ijk - ko, ijk + 1 - ko,
                          ijk + ko, ijk + 1 + ko,
                          ijk, ijk + jo, ijk - 1, ijk + jo - 1, ijk + 1, ijk + jo + 1, ijk - ko, ijk + jo - ko,
                          ijk + ko, ijk + jo + ko,
                          ijk, ijk + ko, ijk - 1, ijk - 1 + ko, ijk + 1, ijk + 1 + ko, ijk - jo, ijk - jo + ko,
                          ijk + jo, ijk + jo + ko};
    Dual<1> in[NSG];
#pragma unroll
    for (int m = 0; m < NSG; m++) {
        const int f = m / 10;
        in[m].v = base.f[f][at[m]];
        in[m].d[0] = mode == 0 ? tan.f[f][at[m]] : (m == q0 ? 1.0 : 0.0);
    }
    const long ij = IDX2(b, i, j);
    Dual<1> g = smag_cell(in, dip[ij], djp[ij], dkp[b.off1k + k - 1], hijp[ij], hjip[ij], csles, vdd[ijk]);
    if (mode == 0) {
        out[ijk] = g.d[0];
    } else {
        const double c = lam[ijk] * g.d[0];
        if (c != 0.) atomicAdd(bar.f[q0 / 10] + at[q0], c);
    }
}

// wall ghosts written by set_virt_bc (set_virt_bc_block.F), linearised:
// ghost = +/- interior (the log-law branch shifts by a constant of the
// running means; the laminar one reflects), for u and w on the WALL y
// sides.  mode 0: tangent ghost = s * tangent interior; mode 1: adjoint
// interior += s * adjoint ghost, adjoint ghost = 0.  blockIdx.z: 0 u, 1 w.
__global__ void k_vbc_lin(const BlkDev *__restrict__ blk, int mode, double *__restrict__ fu, double *__restrict__ fw,
                          const double *__restrict__ tws_u, const double *__restrict__ twn_u,
                          const double *__restrict__ tws_w, const double *__restrict__ twn_w,
                          const long *__restrict__ off_ki, const double *__restrict__ dju,
                          const double *__restrict__ djp, const double *__restrict__ rho, double visc, double ylam)
{
    const BlkDev b = blk[blockIdx.y];
    const int n0 = b.n[0], n1 = b.n[1], n2 = b.n[2];
    const long jo = n0, ko = (long)n0 * n1;
    const int comp = blockIdx.z >> 1, side = 3 + (blockIdx.z & 1);
    if (b.bc[side - 1] != LES_BCT_WALL_D) return;
    double *f = comp == 0 ? fu : fw;
    const double *tw = comp == 0 ? (side == 3 ? tws_u : twn_u) : (side == 3 ? tws_w : twn_w);
    const double *dj = comp == 0 ? dju : djp;
    const int jg = side == 3 ? 1 : n1, jn = side == 3 ? 2 : n1 - 1, k1 = side == 3 ? 2 : n1;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < (long)n0 * n2; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % n0) + 1, k = (int)(q / n0) + 1;
        const long g = b.off3 + (i - 1) + jo * (jg - 1) + ko * (k - 1), nx = g + (jn - jg) * jo;
        const double twv = tw[off_ki[blockIdx.y] + (k - 1) + (long)n2 * (i - 1)];
        // the face density of the forward kernels (interior i, k: the i-1
        // neighbours for u, the k-1 ones for w)
        const long o = comp == 0 ? 1 : ko;
        const bool in = comp == 0 ? i > 1 : k > 1;
        const double r = in ? 0.25 * (rho[g] + rho[nx] + rho[g - o] + rho[nx - o]) : 0.5 * (rho[g] + rho[nx]);
        const double dist = 0.5 * dj[b.off2 + (i - 1) + (long)n0 * (k1 - 1)];
        const double yp = dist * sqrt(fabs(twv) / r) * r / visc;
        const double sgn = yp > ylam ? 1.0 : -1.0;
        if (mode == 0) {
            f[g] = sgn * f[nx];
        } else {
            atomicAdd(f + nx, sgn * f[g]);  // nx is shared by both sides when n1 == 3
            f[g] = 0.0;
        }
    }
}

// ---------------------------------------------------- linear transposes
// swap_sc transposed: unpack^T then pack^T (k_halo_pack / k_halo_unpack)
__global__ void k_halo_unpack_t(const FaceDev *__restrict__ fc, double *__restrict__ bar,
                                double *__restrict__ wbar)
{
    const FaceDev f = fc[blockIdx.y];
    long n = (long)f.nj * f.nk;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        long k = q / f.nj, j = q - k * f.nj;
        if (face_skips(f, j, k)) {
            wbar[f.pwoff + q] = 0.;
            continue;
        }
        long g = f.gh + f.jo * j + f.ko * k;
        wbar[f.pwoff + q] = bar[g];
        bar[g] = 0.;
    }
}

__global__ void k_halo_pack_t(const FaceDev *__restrict__ fc, double *__restrict__ bar,
                              const double *__restrict__ wbar)
{
    const FaceDev f = fc[blockIdx.y];
    long n = (long)f.nj * f.nk;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        long k = q / f.nj, j = q - k * f.nj;
        double v = wbar[f.woff + q];
        if (v != 0.) atomicAdd(bar + f.pk + f.jo * j + f.ko * k, v);
    }
}

// extrap_p transposed (k_extrap_p: sides 1..6 in turn, ghost := inner)
__global__ void k_extrap_p_t(const BlkDev *__restrict__ blk, double *__restrict__ bar)
{
    const BlkDev b = blk[blockIdx.x];
    const int co[2][4] = {{0, 2, 1, 1}, {0, 3, 3, 2}};
    long st[4] = {0, 1, b.n[0], (long)b.n[0] * b.n[1]};
    int nn[4] = {0, b.n[0], b.n[1], b.n[2]};
    for (int s = 6; s >= 1; s--) {
        int bc = b.bc[s - 1];
        if (bc != LES_BCT_PERIODIC_D && bc != LES_BCT_INTERFACE_D) {
            int d1 = (s + 1) / 2, d2 = co[0][d1], d3 = co[1][d1];
            long base = (s % 2 == 1) ? 0 : st[d1] * (nn[d1] - 1);
            long io1 = (s % 2 == 0) ? -st[d1] : st[d1];
            long n = (long)nn[d2] * nn[d3];
            for (long q = threadIdx.x; q < n; q += blockDim.x) {
                long kk = q / nn[d2], jj = q - kk * nn[d2];
                long g = b.off3 + base + st[d2] * jj + st[d3] * kk;
                bar[g + io1] += bar[g];
                bar[g] = 0.;
            }
        }
        __syncthreads();
    }
}

// p_ref_subtract transposed: the reference point takes minus the sum of all
// adjoints (every point had the reference value subtracted)
__global__ void k_pref_t(const BlkDev *__restrict__ blk, double *__restrict__ bar, long n)
{
    double v[1] = {0.};
    for (long q = threadIdx.x; q < n; q += blockDim.x) v[0] += bar[q];
    __shared__ double tot[1];
    block_reduce_store<1>(v, tot);
    __syncthreads();
    if (threadIdx.x == 0) {
        const BlkDev b = blk[0];
        bar[b.off3 + 1 + (long)b.n[0] * (1 + (long)b.n[1])] -= tot[0];
    }
}

// sour_p transposed (k_sour_p: s = -ddtime (gef - gwf + gnf - gsf + grf - glf) - ...)
__global__ void k_sour_p_t(const BlkDev *__restrict__ blk, double dtime, const double *__restrict__ rdiv,
                           const double *__restrict__ rdju, const double *__restrict__ didjp,
                           const double *__restrict__ dkp, const double *__restrict__ rhonp1,
                           const double *__restrict__ sbar, double *__restrict__ ubar,
                           double *__restrict__ vbar, double *__restrict__ wbar)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long p = decode_interior(b, q, i, j, k);
    double sb = sbar[p];
    if (sb == 0.) return;
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    double ddtime = 2.0 / (3.0 * dtime) * 0.5;
    double dkpk = dkp[b.off1k + k - 1];
    double cw = rdju[IDX2(b, i, j)] * dkpk * (rhonp1[p] + rhonp1[p - 1]);
    double ce = rdju[IDX2(b, i + 1, j)] * dkpk * (rhonp1[p] + rhonp1[p + 1]);
    double cs = rdiv[IDX2(b, i, j)] * dkpk * (rhonp1[p] + rhonp1[p - jo]);
    double cn = rdiv[IDX2(b, i, j + 1)] * dkpk * (rhonp1[p] + rhonp1[p + jo]);
    double cr = didjp[IDX2(b, i, j)];
    double cl = cr * (rhonp1[p] + rhonp1[p - ko]), crr = cr * (rhonp1[p] + rhonp1[p + ko]);
    double a = ddtime * sb;
    atomicAdd(ubar + p, a * cw);
    atomicAdd(ubar + p + 1, -a * ce);
    atomicAdd(vbar + p, a * cs);
    atomicAdd(vbar + p + jo, -a * cn);
    atomicAdd(wbar + p, a * cl);
    atomicAdd(wbar + p + ko, -a * crr);
}

// uvw_adv transposed: u = u_int - 1.5 dt dp / rhou on the points it writes;
// the consumed adjoint moves to u_int and p, the point's adjoint is cleared
__global__ void k_uvw_adv_t(const BlkDev *__restrict__ blk, int ivar, double dtime,
                            const double *__restrict__ dg, const double *__restrict__ rp,
                            const double *__restrict__ dkw, double *__restrict__ ubar,
                            double *__restrict__ uibar, const double *__restrict__ rho,
                            double *__restrict__ pbar)
{
    const BlkDev b = blk[blockIdx.y];
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= b.ncell) return;
    int i, j, k;
    long ijk = decode_interior(b, q, i, j, k);
    auto per = [](int bc) { return bc == LES_BCT_PERIODIC_D || bc == LES_BCT_INTERFACE_D; };
    int istr = (ivar == 1 && !per(b.bc[0])) ? 3 : 2;
    int jstr = (ivar == 2 && !per(b.bc[2])) ? 3 : 2;
    int kstr = (ivar == 3 && !per(b.bc[4])) ? 3 : 2;
    if (ivar == 3) istr = jstr;
    if (i < istr || j < jstr || k < kstr) return;
    double ub = ubar[ijk];
    ubar[ijk] = 0.;
    uibar[ijk] += ub;
    double ddtime = 1.5 * dtime;
    long jo = b.n[0], ko = (long)b.n[0] * b.n[1];
    long ijkw;
    double c;
    if (ivar != 3) {
        ijkw = ijk - (ivar == 1 ? 1 : jo);
        c = ddtime / (0.5 * (rho[ijk] + rho[ijkw])) / dg[IDX2(b, i, j)];
    } else {
        ijkw = ijk - ko;
        c = ddtime / (0.5 * (rho[ijk] + rho[ijkw])) / (rp[IDX2(b, i, j)] * dkw[b.off1k + k - 1]);
    }
    atomicAdd(pbar + ijk, -c * ub);
    atomicAdd(pbar + ijkw, c * ub);
}

// mean wall shear stress over the wall points of the y sides:
// visc * u / (0.5 dju) per wall point (the laminar branch); out[0] += sum,
// and its gradient coef into ubar when ubar != null
__global__ void k_wall_shear(const BlkDev *__restrict__ blk, const double *__restrict__ dju, double visc,
                             const double *__restrict__ u, double coef, double *__restrict__ ubar,
                             double *__restrict__ sum)
{
    const BlkDev b = blk[blockIdx.y];
    long n = (long)(b.n[0] - 2) * (b.n[2] - 2);
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    double v[1] = {0.};
    if (q < 2 * n) {
        int side = q >= n;
        long r = q - side * n;
        int i = (int)(r % (b.n[0] - 2)) + 2, k = (int)(r / (b.n[0] - 2)) + 2;
        if (b.bc[2 + side] == LES_BCT_WALL_D) {
            int j = side ? b.n[1] - 1 : 2;
            long ijk = b.off3 + (i - 1) + (long)b.n[0] * (j - 1) + (long)b.n[0] * b.n[1] * (k - 1);
            double g = visc / (0.5 * dju[IDX2(b, i, j)]);
            v[0] = g * u[ijk];
            if (ubar) ubar[ijk] += coef * g;
        }
    }
    __shared__ double t[1];
    block_reduce_store<1>(v, t);
    __syncthreads();
    if (threadIdx.x == 0 && sum) atomicAdd(sum, t[0]);
}

// wall points counted by k_wall_shear
__global__ void k_fill_d(double *__restrict__ a, double v, long n)
{
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) a[q] = v;
}

// ================================================================ launchers
namespace les {

static inline unsigned nbk_(long n, int t) { return (unsigned)((n + t - 1) / t); }

void launch_upred_lin(const BlkDev *blk, int nb, long maxcell, int iva, int mode, int q0, const UIntArgs &a,
                      const PredRefs &base, const PredRefs &tan, const PredBars &bar, const double *lam_u,
                      const double *lam_h, double *out_u, double *out_h, double dtime, double visc,
                      double ylaminar, double kappa, double cwfun, cudaStream_t st)
{
    k_upred_lin<<<dim3(nbk_(maxcell, 128), nb), 128, 0, st>>>(blk, iva, mode, q0, a, base, tan, bar, lam_u, lam_h,
                                                              out_u, out_h, dtime, visc, ylaminar, kappa, cwfun);
    count_launch(1);
}

void launch_wpred_lin(const BlkDev *blk, int nb, long maxcell, int mode, int q0, const WIntArgs &a,
                      const PredRefs &base, const PredRefs &tan, const PredBars &bar, const double *lam_u,
                      const double *lam_h, double *out_u, double *out_h, double dtime, double visc,
                      double ylaminar, double kappa, double cwfun, cudaStream_t st)
{
    k_wpred_lin<<<dim3(nbk_(maxcell, 128), nb), 128, 0, st>>>(blk, mode, q0, a, base, tan, bar, lam_u, lam_h,
                                                              out_u, out_h, dtime, visc, ylaminar, kappa, cwfun);
    count_launch(1);
}

void launch_take(const BlkDev *blk, int nb, long maxcell, int which, const double *src, double *dst,
                 double *zero_src, cudaStream_t st)
{
    k_take<<<dim3(nbk_(maxcell, 256), nb), 256, 0, st>>>(blk, which, src, dst, zero_src);
    count_launch(1);
}

void launch_halo_t(const FaceDev *faces, int nface, long maxface, double *bar, double *wbar, cudaStream_t st)
{
    if (nface == 0) return;
    unsigned gx = nbk_(maxface, 256);
    if (gx > 64) gx = 64;
    k_halo_unpack_t<<<dim3(gx, nface), 256, 0, st>>>(faces, bar, wbar);
    k_halo_pack_t<<<dim3(gx, nface), 256, 0, st>>>(faces, bar, wbar);
    count_launch(2);
}

void launch_extrap_p_t(const BlkDev *blk, int nb, double *bar, cudaStream_t st)
{
    k_extrap_p_t<<<nb, 256, 0, st>>>(blk, bar);
    count_launch(1);
}

void launch_pref_t(const BlkDev *blk, double *bar, long n, cudaStream_t st)
{
    k_pref_t<<<1, 1024, 0, st>>>(blk, bar, n);
    count_launch(1);
}

void launch_sour_p_t(const BlkDev *blk, int nb, long maxcell, double dtime, const double *rdiv,
                     const double *rdju, const double *didjp, const double *dkp, const double *rhonp1,
                     const double *sbar, double *ubar, double *vbar, double *wbar, cudaStream_t st)
{
    k_sour_p_t<<<dim3(nbk_(maxcell, 256), nb), 256, 0, st>>>(blk, dtime, rdiv, rdju, didjp, dkp, rhonp1, sbar,
                                                             ubar, vbar, wbar);
    count_launch(1);
}

void launch_uvw_adv_t(const BlkDev *blk, int nb, long maxcell, int ivar, double dtime, const double *dg,
                      const double *rp, const double *dkw, double *ubar, double *uibar, const double *rho,
                      double *pbar, cudaStream_t st)
{
    k_uvw_adv_t<<<dim3(nbk_(maxcell, 256), nb), 256, 0, st>>>(blk, ivar, dtime, dg, rp, dkw, ubar, uibar, rho,
                                                              pbar);
    count_launch(1);
}

void launch_wall_shear(const BlkDev *blk, int nb, long maxik, const double *dju, double visc, const double *u,
                       double coef, double *ubar, double *sum, cudaStream_t st)
{
    k_wall_shear<<<dim3(nbk_(2 * maxik, 256), nb), 256, 0, st>>>(blk, dju, visc, u, coef, ubar, sum);
    count_launch(1);
}

void launch_sgs_lin(const BlkDev *blk, int nb, long maxcell, int mode, int q0, const PredRefs &base,
                    const PredRefs &tan, const PredBars &bar, const double *lam, double *out, const double *dip,
                    const double *djp, const double *dkp, const double *hijp, const double *hjip, const double *vdd,
                    double csles, cudaStream_t st)
{
    k_sgs_lin<<<dim3(nbk_(maxcell, 128), nb), 128, 0, st>>>(blk, mode, q0, base, tan, bar, lam, out, dip, djp, dkp,
                                                            hijp, hjip, vdd, csles);
    count_launch(1);
}

void launch_vbc_lin(const BlkDev *blk, int nb, long maxik, int mode, double *fu, double *fw, const double *tws_u,
                    const double *twn_u, const double *tws_w, const double *twn_w, const long *off_ki,
                    const double *dju, const double *djp, const double *rho, double visc, double ylam,
                    cudaStream_t st)
{
    unsigned g = nbk_(maxik, 128);
    k_vbc_lin<<<dim3(g > 1024 ? 1024 : g, nb, 4), 128, 0, st>>>(blk, mode, fu, fw, tws_u, twn_u, tws_w, twn_w,
                                                                off_ki, dju, djp, rho, visc, ylam);
    count_launch(1);
}

void launch_fill_d(double *a, double v, long n, cudaStream_t st)
{
    unsigned g = nbk_(n, 256);
    k_fill_d<<<g > 2048 ? 2048 : g, 256, 0, st>>>(a, v, n);
    count_launch(1);
}

} // namespace les
