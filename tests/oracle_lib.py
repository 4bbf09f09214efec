"""ctypes access to the CPU parity oracle (oracle/_build/liblester_oracle.so).

Test infrastructure only: the oracle is the checker, never the thing
measured or shipped.  It is built from oracle/ by ``make -C oracle``.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
ORACLE_DIR = ROOT / "oracle"
ORACLE_SO = ORACLE_DIR / "_build" / "liblester_oracle.so"

_lib = None


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR)], check=True)
    return ORACLE_SO


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build_oracle()
        _lib = C.CDLL(str(ORACLE_SO))
        _lib.orc_create.restype = C.c_void_p
        _lib.orc_npts_all.restype = C.c_double
        for name in dir(_lib):
            pass
    return _lib


def P(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


class MgCtrl(C.Structure):
    _fields_ = [("nummgits", C.c_int), ("numpre", C.c_int), ("numpost", C.c_int),
                ("numcits", C.c_int), ("meth_cycle", C.c_int), ("meth_smooth", C.c_int),
                ("meth_csolve", C.c_int), ("tolf", C.c_double), ("relax_pmg", C.c_double),
                ("relax_pmgc", C.c_double), ("compat", C.c_int)]


class Oracle:
    """One oracle context for a grid.Case (levels capped like the case)."""

    def __init__(self, case):
        self.case = case
        nb, n, bc, l1, l2 = case.oracle_args()
        st = C.c_int()
        self._keep = (n, bc, l1, l2)
        self.ctx = C.c_void_p(lib().orc_create(nb, n.ctypes.data_as(C.c_void_p),
                                               bc.ctypes.data_as(C.c_void_p),
                                               l1.ctypes.data_as(C.c_void_p),
                                               l2.ctypes.data_as(C.c_void_p), case.maxmgl,
                                               case.nummgl, C.byref(st)))
        if st.value != 0:
            raise RuntimeError(f"orc_create failed: {st.value}")

    def __del__(self):
        try:
            lib().orc_destroy(self.ctx)
        except Exception:
            pass

    def sizes(self):
        out = (C.c_long * 9)()
        lib().orc_sizes(self.ctx, out)
        return list(out)

    def block_info(self, ilev, iblk):
        n = (C.c_int * 3)()
        m = (C.c_int * 3)()
        o = (C.c_long * 7)()
        lib().orc_block_info(self.ctx, ilev, iblk, n, m, o)
        return tuple(n), tuple(m), tuple(o)

    def set_loop_bound(self, ivar):
        lib().orc_set_loop_bound(self.ctx, ivar)

    def npts_all(self, ilev):
        return lib().orc_npts_all(self.ctx, ilev)

    def set_jumble(self, j):
        lib().orc_set_jumble(self.ctx, j)

    def get_jumble(self):
        return lib().orc_get_jumble(self.ctx)

    def swap_sc(self, igrid, var, mg_or_sg=1):
        lib().orc_swap_sc(self.ctx, igrid, P(var), mg_or_sg)

    def comp_metric(self, x, y, z, gotrad=0):
        c = self.case
        metric = np.zeros(35 * c.n2)
        dkp = np.zeros(c.n1k)
        dkw = np.zeros(c.n1k)
        lib().orc_comp_metric(self.ctx, P(x), P(y), P(z), P(metric), P(dkp), P(dkw), gotrad)
        return metric.reshape(35, c.n2), dkp, dkw

    def coeff_p(self, m, dkp, dkw, a):
        lib().orc_coeff_p(self.ctx, *map(P, (m["diu"], m["djv"], m["rdiv"], m["rdju"],
                                             m["didjp"], m["rp"], dkp, dkw)), *map(P, a))

    def sour_p(self, dtime, m, dkp, dkw, u, v, w, rho, rhonp1, out4):
        lib().orc_sour_p(self.ctx, C.c_double(dtime),
                         *map(P, (m["diu"], m["djv"], m["rdiv"], m["rdju"], m["didjp"], dkp,
                                  m["rdidjp"], dkw, u, v, w, rho, rhonp1)), *map(P, out4))

    def norms(self, ilev, mg_or_sg, a, x, b, residu):
        out = np.zeros(4)
        lib().orc_norms(self.ctx, ilev, mg_or_sg, *map(P, a), P(x), P(b), P(residu), P(out))
        return tuple(out)

    def restriction(self, ilev, f, f1):
        lib().orc_restriction(self.ctx, ilev, P(f), P(f1))

    def prolongation(self, ilev, f):
        lib().orc_prolongation(self.ctx, ilev, P(f))

    def sporlx(self, ilev, a, f, b, omega, soltol, norms4):
        io = np.array(norms4, dtype=np.float64)
        lib().orc_sporlx(self.ctx, ilev, *map(P, a), P(f), P(b), C.c_double(omega),
                         C.c_double(soltol), P(io))
        return tuple(io)

    def lmg_solve(self, ctrl: MgCtrl, a, f, b, residu):
        out = np.zeros(5)
        lib().orc_lmg_solve(self.ctx, C.byref(ctrl), *map(P, a), P(f), P(b), P(residu), P(out))
        return out

    def extrap_p(self, p):
        lib().orc_extrap_p(self.ctx, P(p))

    def p_ref_subtract(self, p):
        lib().orc_p_ref_subtract(self.ctx, P(p))

    def uvw_adv(self, ivar, dtime, dg, rp, dkw, u, u_int, rho, p):
        lib().orc_uvw_adv(self.ctx, ivar, C.c_double(dtime), *map(P, (dg, rp, dkw, u, u_int, rho,
                                                                       p)))

    def swap_rhos(self, rho, rhonp1, rhonm1):
        lib().orc_swap_rhos(self.ctx, P(rho), P(rhonp1), P(rhonm1))

    def search_lib(self, sc1, rhonp1, alpha, rho, rholo, rhohi):
        lib().orc_search_lib(self.ctx, P(sc1), P(rhonp1), C.c_double(alpha), P(rho),
                             C.c_double(rholo), C.c_double(rhohi))

    def slipbc(self, dtime, djp, u, v, v_int, w, sc1, rho, p):
        lib().orc_slipbc(self.ctx, C.c_double(dtime), *map(P, (djp, u, v, v_int, w, sc1, rho, p)))

    def subgrid(self, model, csles, gotrad, gam, gamsc1, u, v, w, sc1, sc1var, sc1dis, vdd, m,
                dkp, dkw, alpha=0.0):
        lib().orc_subgrid(self.ctx, model, C.c_double(csles), gotrad, C.c_double(alpha),
                          *map(P, (gam, gamsc1, u, v, w, sc1, sc1var, sc1dis, vdd, m["dip"],
                                   m["diu"], m["djp"], m["djv"], dkp, dkw, m["hijp"], m["hjip"],
                                   m["hkip"], m["hkjp"], m["rp"])))


def mgctrl(nummgits=5, numpre=1, numpost=1, numcits=20, meth_cycle=1, tolf=5e-13, relax=1.6,
           compat=0):
    c = MgCtrl()
    c.compat = compat
    c.nummgits, c.numpre, c.numpost, c.numcits = nummgits, numpre, numpost, numcits
    c.meth_cycle, c.meth_smooth, c.meth_csolve = meth_cycle, 1, 0
    c.tolf, c.relax_pmg, c.relax_pmgc = tolf, relax, relax
    return c


def _flat_metric(m: dict) -> np.ndarray:
    from fortranutils_gb300 import lester as L
    return np.ascontiguousarray(np.stack([m[n] for n in L.METRIC_NAMES]))


def _orc_predictor_methods():
    D = C.c_double

    def set_uv_int(self, iva, dtime, iststep, k, u, v, w, p, rho, rhonp1, gam, u_int, hu, m, dkp,
                   dkw, tw):
        flat = _flat_metric(m)  # kept alive across the call
        lib().orc_set_uv_int(self.ctx, iva, D(dtime), iststep, D(k["visc"]), D(k["ylaminar"]),
                             D(k["kappa"]), D(k["cwfun"]),
                             *map(P, (u, v, w, p, rho, rhonp1, gam, u_int, hu, flat, dkp,
                                      dkw, *tw)))

    def set_w_int(self, dtime, iststep, k, u, v, w, p, rho, rhonp1, gam, w_int, hw, m, dkp, dkw,
                  tw):
        flat = _flat_metric(m)
        lib().orc_set_w_int(self.ctx, D(dtime), iststep, D(k["visc"]), D(k["ylaminar"]),
                            D(k["kappa"]), D(k["cwfun"]),
                            *map(P, (u, v, w, p, rho, rhonp1, gam, w_int, hw, flat, dkp,
                                     dkw, *tw)))

    def set_gamsc1_bc(self, visc, sc1, gamsc1, gamlam, m, dkp):
        flat = _flat_metric(m)
        lib().orc_set_gamsc1_bc(self.ctx, D(visc), P(sc1), P(gamsc1), P(gamlam), P(flat), P(dkp))

    def set_sc1(self, dtime, m, dkp, dkw, u, v, w, sc1, hsc1, rho, gamsc1, gamlam):
        flat = _flat_metric(m)
        lib().orc_set_sc1(self.ctx, D(dtime), P(flat), *map(P, (dkp, dkw, u, v, w, sc1,
                                                                           hsc1, rho, gamsc1,
                                                                           gamlam)))

    def set_sc1_bc(self, f):
        lib().orc_set_sc1_bc(self.ctx, P(f))

    def set_sc1var(self, sc1, sc1var, m, dkp, dkw):
        flat = _flat_metric(m)
        lib().orc_set_sc1var(self.ctx, P(sc1), P(sc1var), P(flat), P(dkp), P(dkw))

    for f in (set_uv_int, set_w_int, set_gamsc1_bc, set_sc1, set_sc1_bc, set_sc1var):
        setattr(Oracle, f.__name__, f)


_orc_predictor_methods()


class OrcPhys(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dtime visc csles rholo rhohi alpha ylaminar kappa "
                                           "cwfun aplus").split()] + [("model", C.c_int),
                                                                      ("gotrad", C.c_int)]


class OrcFields(C.Structure):
    _fields_ = ([(n, C.c_void_p) for n in (
        "u v w sc1 rho rhonp1 rhonm1 u_int v_int w_int hn_u hn_v hn_w hn_sc1 gam gamsc1 gamlam "
        "sc1var sc1dis vd_damping temperature drhonp1dt srhot srhoux p s res ap aw ae as an al "
        "ar metric dkp dkw").split()] + [("tw", C.c_void_p * 12)])


def phys_from_ctrl(ctrl, gotrad=0) -> OrcPhys:
    k = OrcPhys()
    for n in "dtime visc csles rholo rhohi alpha ylaminar kappa cwfun aplus model".split():
        setattr(k, n, getattr(ctrl, n))
    k.gotrad = gotrad
    return k


def mgctrl_from_ctrl(ctrl) -> MgCtrl:
    return mgctrl(ctrl.nummgits, ctrl.numpre, ctrl.numpost, ctrl.numcits, ctrl.meth_cycle,
                  ctrl.tolf, ctrl.relax_pmg)


def _orc_step(self, mg: MgCtrl, k: OrcPhys, istep: int, iststep: int, state) -> None:
    """orc_step on a numpy State (fortranutils_gb300.state)."""
    from fortranutils_gb300 import state as S
    flat = _flat_metric(state["metric"])
    f = OrcFields()
    for n in S.FIELDS3 + S.FIELDSM:
        setattr(f, n, P(state[n]).value)
    f.metric = P(flat).value
    f.dkp = P(state["dkp"]).value
    f.dkw = P(state["dkw"]).value
    for q, n in enumerate(S.TW):
        f.tw[q] = P(state[n]).value
    lib().orc_step(self.ctx, C.byref(mg), C.byref(k), istep, iststep, C.byref(f))


Oracle.step = _orc_step


# ---- convective outflow / fixed inflow (oracle/orc_outflow.c) ------------
def _orc_conv_exitbc(self, task, iva, dtime, rho, rhonp1, u, v, w, u_int, v_int, w_int, hu, hv, hw,
                     metric: dict, dkp, dkw) -> None:
    flat = _flat_metric(metric)
    lib().orc_conv_exitbc(self.ctx, int(task), int(iva), C.c_double(dtime),
                          *map(P, (rho, rhonp1, u, v, w, u_int, v_int, w_int, hu, hv, hw, flat, dkp, dkw)))


def _orc_mass_change(self, dtime, rho, rhonp1, rdidjp, dkw) -> float:
    lib().orc_mass_change.restype = C.c_double
    return lib().orc_mass_change(self.ctx, C.c_double(dtime), P(rho), P(rhonp1), P(rdidjp), P(dkw))


def _orc_fixed_inlet(self, inlet, uprof, vprof, seed, step, rholo, rhohi, u, v, w, sc1, rho, u_int,
                     v_int, w_int) -> None:
    ib = (C.c_int * 4)(*inlet)
    lib().orc_fixed_inlet(self.ctx, ib, P(uprof), P(vprof), C.c_ulonglong(seed), int(step),
                          C.c_double(rholo), C.c_double(rhohi),
                          *map(P, (u, v, w, sc1, rho, u_int, v_int, w_int)))


def _orc_set_inlet(self, inlet, uprof, vprof, seed) -> None:
    ib = (C.c_int * 4)(*inlet)
    lib().orc_set_inlet(self.ctx, ib, P(uprof), P(vprof), len(uprof), C.c_ulonglong(seed))


Oracle.conv_exitbc = _orc_conv_exitbc
Oracle.mass_change = _orc_mass_change
Oracle.fixed_inlet = _orc_fixed_inlet
Oracle.set_inlet = _orc_set_inlet


def _orc_recycling(self, step, inblock, inlet, rhohi, u, v, w, sc1, rho, u_int, v_int, w_int, prof, means):
    ib = (C.c_int * 4)(*inlet)
    lib().orc_recycling(self.ctx, int(step), int(inblock), ib, C.c_double(rhohi),
                        *map(P, (u, v, w, sc1, rho, u_int, v_int, w_int)), *map(P, prof), *map(P, means))


Oracle.recycling = _orc_recycling


def _orc_statistics(self, no_sam, u, v, w, p, rho, sc1, sc1var, gam, outs: dict) -> None:
    from fortranutils_gb300 import lester as L
    arr = (C.c_void_p * 16)(*[P(outs[n]).value for n in L.STAT_NAMES])
    lib().orc_statistics(self.ctx, int(no_sam), *map(P, (u, v, w, p, rho, sc1, sc1var, gam)), arr)


Oracle.statistics = _orc_statistics
