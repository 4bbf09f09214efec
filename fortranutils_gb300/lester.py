"""Python binding of liblester_gpu.so (include/lester_gpu.h).

The functions keep the reference's subroutine names and argument order
(code/step.F calls them); arrays may be torch CUDA tensors (used in place on
the device) or numpy arrays (copied in and out by the library).  Scalars are
passed by reference, as Fortran does.  Every call checks the returned status
and raises ``LesterError`` with the library's message.

There is no CPU fallback: if the shared library is missing this module
raises at import time.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build

LES_MAXBL = 64
LES_MAXMGL = 16

BCT_WALL, BCT_ZERO_GRAD, BCT_CONVECTIVE, BCT_FIXED = 1, 2, 3, 4
BCT_TRACTION, BCT_PERIODIC, BCT_INTERFACE = 6, 12, 13
SV_U, SV_V, SV_W, SV_P, SV_SC1 = 1, 2, 3, 4, 5
PSOLVE_REFERENCE, PSOLVE_FP64, PSOLVE_MIXED = 0, 1, 2

ERRORS = {
    -1: "LES_ERR_NOT_INIT", -2: "LES_ERR_GEOM", -3: "LES_ERR_ARG", -4: "LES_ERR_CUDA",
    -5: "LES_ERR_NOMEM", -6: "LES_ERR_NONFINITE", -7: "LES_ERR_NOT_CONVERGED",
    -8: "LES_ERR_STRUCTURE", -9: "LES_ERR_TIMEOUT", -10: "LES_ERR_SIZE",
}


class LesterError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Geom(C.Structure):
    _fields_ = [
        ("numbl", C.c_int), ("maxmgl", C.c_int), ("nummgl", C.c_int), ("gotrad", C.c_int),
        ("bl_nijkp1", (C.c_int * 3) * LES_MAXBL), ("bl_bc", (C.c_int * 6) * LES_MAXBL),
        ("bl2bl", (C.c_int * 6) * LES_MAXBL), ("bl2side", (C.c_int * 6) * LES_MAXBL),
    ]


class Ctrl(C.Structure):
    _fields_ = [
        ("dtime", C.c_double), ("visc", C.c_double), ("csles", C.c_double),
        ("rholo", C.c_double), ("rhohi", C.c_double), ("alpha", C.c_double),
        ("ylaminar", C.c_double), ("kappa", C.c_double), ("cwfun", C.c_double),
        ("aplus", C.c_double), ("model", C.c_int),
        ("nummgits", C.c_int), ("numpre", C.c_int), ("numpost", C.c_int),
        ("numcits", C.c_int), ("meth_cycle", C.c_int),
        ("tolf", C.c_double), ("relax_pmg", C.c_double), ("relax_pmgc", C.c_double),
        ("psolve", C.c_int), ("rtol", C.c_double), ("max_outer", C.c_int),
        ("rb_sweeps", C.c_int), ("rb_coarse", C.c_int), ("rb_omega", C.c_double),
        ("exact", C.c_int), ("rb_matfree", C.c_int), ("mg_tail", C.c_int), ("krylov", C.c_int),
        ("rb_line", C.c_int), ("autotune", C.c_int), ("phys32", C.c_int), ("step_graph", C.c_int),
        ("sc1_sweep", C.c_int), ("wait_limit", C.c_int), ("p_guess", C.c_int), ("rb_tile", C.c_int),
    ]


class Sizes(C.Structure):
    _fields_ = [("nummgl", C.c_int), ("n3_sg", C.c_long), ("n3_mg", C.c_long), ("n2", C.c_long),
                ("n1k", C.c_long), ("nxy", C.c_long), ("nz", C.c_long), ("n2_ki", C.c_long),
                ("n2_jk", C.c_long)]


def default_ctrl(**kw) -> Ctrl:
    """Controls with the reference defaults (code/defaults.F:59-71, const.inc)."""
    c = Ctrl()
    c.dtime = 1e-3
    c.visc = 1.0 / 2800.0
    c.csles = 0.1
    c.rholo = 1.0
    c.rhohi = 1.0
    c.alpha = 0.0
    c.ylaminar = 11.3
    c.kappa = 0.41
    c.cwfun = 5.2 * 0.41
    c.aplus = 25.0
    c.model = 1
    c.nummgits = 5
    c.numpre = 1
    c.numpost = 1
    c.numcits = 20
    c.meth_cycle = 1
    c.tolf = 5e-13
    c.relax_pmg = 1.6
    c.relax_pmgc = 1.6
    c.psolve = PSOLVE_REFERENCE
    c.rtol = 1e-8
    c.max_outer = 200
    c.rb_sweeps = 3
    c.rb_coarse = 20
    c.rb_omega = 1.5
    c.exact = 1
    c.rb_matfree = 1
    c.mg_tail = 4096
    c.krylov = 2
    for k, v in kw.items():
        setattr(c, k, v)
    return c


_lib = None


def lib() -> C.CDLL:
    """Load the in-tree shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        path = _build.lib_path()
        if not path.exists():
            raise ImportError(f"{path} is missing: run fortranutils_gb300.build.build() first")
        _lib = C.CDLL(str(path))
        _lib.lester_gpu_last_error.restype = C.c_char_p
        _lib.lester_gpu_get_stream.restype = C.c_void_p
        _lib.lester_gpu_launch_count.restype = C.c_long
        _lib.lester_gpu_set_stream.argtypes = [C.c_void_p]
    return _lib


def _check(code: int) -> None:
    if code != 0:
        raise LesterError(code, lib().lester_gpu_last_error().decode())


def _p(a):
    """Raw pointer of a float64 contiguous torch tensor or numpy array."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
            raise TypeError("arrays must be contiguous float64")
        return C.c_void_p(a.ctypes.data)
    import torch
    if a.dtype != torch.float64 or not a.is_contiguous():
        raise TypeError("tensors must be contiguous float64")
    return C.c_void_p(a.data_ptr())


def _i(v: int):
    return C.byref(C.c_int(int(v)))


def _d(v: float):
    return C.byref(C.c_double(float(v)))


# ------------------------------------------------------------- lifecycle
def gpu_init(geom: Geom, ctrl: Ctrl, stream: int | None = None) -> None:
    """Initialise; the library then queues its work on ``stream`` (default:
    torch's current stream, so torch ops and library calls stay ordered)."""
    _check(lib().lester_gpu_init(C.byref(geom), C.byref(ctrl)))
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                stream = torch.cuda.current_stream().cuda_stream
        except ImportError:
            pass
    if stream is not None:
        _check(lib().lester_gpu_set_stream(C.c_void_p(stream)))


def gpu_set_ctrl(ctrl: Ctrl) -> None:
    _check(lib().lester_gpu_set_ctrl(C.byref(ctrl)))


def gpu_finalize() -> None:
    _check(lib().lester_gpu_finalize())


def gpu_sizes() -> Sizes:
    s = Sizes()
    _check(lib().lester_gpu_sizes(C.byref(s)))
    return s


def gpu_block_info(ilev: int, iblk: int):
    n = (C.c_int * 3)()
    o = (C.c_long * 5)()
    _check(lib().lester_gpu_block_info(ilev, iblk, n, o))
    return tuple(n), tuple(o)


def gpu_sync() -> None:
    _check(lib().lester_gpu_sync())


def gpu_stream() -> int:
    return lib().lester_gpu_get_stream()


def gpu_set_jumble(j: int) -> None:
    _check(lib().lester_gpu_set_jumble(int(j)))


def gpu_get_jumble() -> int:
    return lib().lester_gpu_get_jumble()


def gpu_launch_count() -> int:
    return lib().lester_gpu_launch_count()


def gpu_solve_stats():
    o = (C.c_double * 6)()
    _check(lib().lester_gpu_solve_stats(o))
    return {"rnorm": o[0], "fnorm": o[1], "enorm": o[2], "vnorm": o[3], "cycles": int(o[4]),
            "relres": o[5]}


def gpu_step_graph_info() -> dict:
    """Steps replayed from the whole-step graph since gpu_init, the solves
    among them the host loop finished, and whether the current fields'
    graph failed to capture (with the reason)."""
    n, h, f = C.c_long(), C.c_long(), C.c_int()
    why = C.create_string_buffer(512)
    _check(lib().lester_gpu_step_graph_info(C.byref(n), C.byref(h), C.byref(f), why, 512))
    return {"replays": n.value, "handovers": h.value, "failed": bool(f.value), "why": why.value.decode()}


def gpu_solver_forms() -> dict:
    """Forms the fast solvers took for the current coefficients."""
    m = C.c_int()
    _check(lib().lester_gpu_solver_forms(C.byref(m)))
    v = m.value
    return {"mf32": bool(v & 1), "df_separable": bool(v & 2), "df_diag_sum": bool(v & 4),
            "direct32": bool(v & 8), "direct64": bool(v & 16)}


def gpu_rb_tiles() -> int:
    """Bit l set: level l was smoothed by the shared-memory red-black tiles."""
    m = C.c_int()
    _check(lib().lester_gpu_rb_tiles(C.byref(m)))
    return m.value


def gpu_step_log(path) -> None:
    """Append one JSON line per lester_step to `path` (None closes)."""
    _check(lib().lester_gpu_step_log(None if path is None else str(path).encode()))


def gpu_tuned(prec: int) -> dict:
    """Settings the autotuner chose for prec 64 (FP64) or 32 (mixed)."""
    d, t, s, tl, ln = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
    om = C.c_double()
    _check(lib().lester_gpu_tuned(int(prec), C.byref(d), C.byref(t), C.byref(s), C.byref(om), C.byref(tl),
                                  C.byref(ln)))
    return {"done": bool(d.value), "rb_threads": t.value, "rb_sweeps": s.value, "rb_omega": om.value,
            "mg_tail": tl.value, "rb_line": ln.value}


def gpu_solve_time() -> float:
    """Device milliseconds of the last fast solve."""
    ms = C.c_double()
    _check(lib().lester_gpu_solve_time(C.byref(ms)))
    return ms.value


# ----------------------------------------------------- reference routines
METRIC_NAMES = ("dip diu div dix rdip rdiv rdix djp dju djv djx rdjp rdju rdjx hijp hjip hkip "
                "hkjp hiju hjiu hkiu hkju hijv hjiv hkiv hkjv rp ru rv didjp rdidjp didju "
                "rdidju djdiv rdjdiv").split()


def swap_sc(ivar1, igrid, var, work=None, mg_or_sg=1):
    _check(lib().lester_swap_sc(_i(ivar1), _i(igrid), _p(var), None, _i(mg_or_sg)))


def comp_metric(x, y, t, metrics: dict, dkp, dkw):
    args = [_p(metrics[n]) for n in METRIC_NAMES]
    _check(lib().lester_comp_metric(_p(x), _p(y), _p(t), *args, _p(dkp), _p(dkw), None, None))


def coeff_p(diu, djv, rdiv, rdju, didjp, rp, dkp, dkw, ap, aw, ae, as_, an, al, ar):
    _check(lib().lester_coeff_p(*map(_p, (diu, djv, rdiv, rdju, didjp, rp, dkp, dkw, ap, aw, ae,
                                          as_, an, al, ar))))


def sour_p(diu, djv, rdiv, rdju, didjp, dkp, rdidjp, dkw, u, v, w, rho, rhonp1, drhonp1dt, s,
           srhot, srhoux):
    _check(lib().lester_sour_p(*map(_p, (diu, djv, rdiv, rdju, didjp, dkp, rdidjp, dkw, u, v, w,
                                         rho, rhonp1, drhonp1dt, s, srhot, srhoux)), None, None))


def lmg_solve(ap, aw, ae, as_, an, al, ar, f, b, residu):
    _check(lib().lester_lmg_solve(*map(_p, (ap, aw, ae, as_, an, al, ar, f, b, residu)), None, None))


def solvers(ap, aw, ae, as_, an, al, ar, f, b, residu):
    _check(lib().lester_solvers(*map(_p, (ap, aw, ae, as_, an, al, ar, f, b, residu)), None, None))


def norms(ilev, mg_or_sg, ap, aw, ae, as_, an, al, ar, x, b, residu):
    o = [C.c_double() for _ in range(4)]
    _check(lib().lester_norms(_i(ilev), _i(mg_or_sg), *map(_p, (ap, aw, ae, as_, an, al, ar, x, b,
                                                                 residu)),
                              *[C.byref(v) for v in o]))
    return tuple(v.value for v in o)


def restriction(ilev, f, f1):
    _check(lib().lester_restriction(_i(ilev), _p(f), _p(f1), None, None))


def prolongation(ilev, f):
    _check(lib().lester_prolongation(_i(ilev), _p(f), None, None))


def sporlx(ilev, ap, aw, ae, as_, an, al, ar, f, b, omega, soltol, norms4):
    o = [C.c_double(v) for v in norms4]
    _check(lib().lester_sporlx(_i(ilev), *map(_p, (ap, aw, ae, as_, an, al, ar, f, b)), None,
                               _i(1), _d(omega), _d(soltol), None, None,
                               *[C.byref(v) for v in o]))
    return tuple(v.value for v in o)


def extrap_p(p):
    _check(lib().lester_extrap_p(_p(p), None, None))


def p_ref_subtract(p):
    _check(lib().lester_p_ref_subtract(_p(p)))


def uvw_adv(ivar1, diu, rp, dkw, u, u_int, rho, p, step=1):
    _check(lib().lester_uvw_adv(_i(ivar1), *map(_p, (diu, rp, dkw, u, u_int, rho, p)), None, None,
                                _i(step)))


def swap_rhos(rho, rhonp1, rhonm1):
    _check(lib().lester_swap_rhos(_p(rho), _p(rhonp1), _p(rhonm1)))


def search_lib(sc1, sc1var, rhonp1, temperature, istep, alpha, rho, rholo, rhohi):
    _check(lib().lester_search_lib(_p(sc1), _p(sc1var), _p(rhonp1), _p(temperature), None, None,
                                   _i(istep), _d(alpha), _p(rho), _d(rholo), _d(rhohi)))


def slipbc(x, y, z, dip, diu, djp, djv, dkp, u, v, v_int, w, sc1, rho, p, step=1):
    _check(lib().lester_slipbc(*map(_p, (x, y, z, dip, diu, djp, djv, dkp, u, v, v_int, w, sc1,
                                         rho, p)), _i(step)))


def subgrid(gam, gamsc1, u, v, w, sc1, rho, sc1var, sc1dis, vd_damping, dip, diu, djp, djv, dkp,
            dkw, hijp, hjip, hkip, hkjp, rp):
    _check(lib().lester_subgrid(*map(_p, (gam, gamsc1, u, v, w, sc1, rho, sc1var, sc1dis,
                                          vd_damping, dip, diu, djp, djv, dkp, dkw, hijp, hjip,
                                          hkip, hkjp, rp)), None, None))


def gpu_prof(enable: bool) -> None:
    _check(lib().lester_gpu_prof(1 if enable else 0))


PROF_RB, PROF_SWEEP = 0, 1


def gpu_prof_read(which: int = PROF_RB):
    """(summed device ms, timed launches) of one timed kernel since
    gpu_prof(True): PROF_RB the level-1 red-black smoother, PROF_SWEEP the
    scalar sweep."""
    ms = C.c_double()
    n = C.c_long()
    _check(lib().lester_gpu_prof_kernel(int(which), C.byref(ms), C.byref(n)))
    return ms.value, n.value


def gpu_xfer_bytes():
    a, b = C.c_long(), C.c_long()
    _check(lib().lester_gpu_xfer_bytes(C.byref(a), C.byref(b)))
    return a.value, b.value


def gpu_set_iststep(iststep: int) -> None:
    _check(lib().lester_gpu_set_iststep(int(iststep)))


def gpu_set_body_force(fu=None, fv=None, fw=None) -> None:
    """Body force per unit volume added to the u, v, w predictors (device
    tensors in the level-1 layout, kept alive by the caller; None = none)."""
    _check(lib().lester_gpu_set_body_force(_p(fu), _p(fv), _p(fw)))


class AdjCfg(C.Structure):
    """include/lester_gpu.h lester_adj_cfg"""
    _fields_ = [("nsteps", C.c_int), ("j_first", C.c_int), ("j_last", C.c_int), ("checkpoint", C.c_int)]


# roles of set_uv_int's metric arguments (code/set_uv_int.F:5-11) and the
# arrays step.F passes for u and for v (code/step.F:307-326)
UV_ROLES = ("dip diu dix rdix djp dju djv djx rdjp rdju didjp didju rdidju hijp hiju hjiu hkiu "
            "hkju rp ru").split()
UV_FOR = {
    1: UV_ROLES,
    2: ("djp djv djx rdjx dip div diu dix rdip rdiv didjp djdiv rdjdiv hjip hjiv hijv hkjv hkiv "
        "rp rv").split(),
}
W_ROLES = "dip diu rdiv djp djv rdju didjp rdidjp hkip hkjp hkiu hkjv rp ru".split()


def set_uv_int(iva, u, v, w, p, rho, rhonp1, gam, u_int, hu, metrics: dict, dkp, dkw, tw_s, tw_n,
               tw_l, tw_r):
    """code/set_uv_int.F; for iva = 2 pass the v field as ``u`` and u as
    ``v`` (step.F does), metrics is the comp_metric dict."""
    mets = [_p(metrics[n]) for n in UV_FOR[iva]]
    _check(lib().lester_set_uv_int(_i(iva), *map(_p, (u, v, w, p, rho, rhonp1, gam, u_int, hu)),
                                   *mets, _p(dkp), _p(dkw), *map(_p, (tw_s, tw_n, tw_l, tw_r)),
                                   None, None))


def set_w_int(u, v, w, p, rho, rhonp1, gam, w_int, hw, metrics: dict, dkp, dkw, tw_sfk, tw_nfk,
              tw_wfk, tw_efk):
    mets = [_p(metrics[n]) for n in W_ROLES]
    _check(lib().lester_set_w_int(*map(_p, (u, v, w, p, rho, rhonp1, gam, w_int, hw)), *mets,
                                  _p(dkp), _p(dkw), *map(_p, (tw_sfk, tw_nfk, tw_wfk, tw_efk)),
                                  None, None))


def set_gamsc1_bc(sc1, gamsc1, gamlam, diu, djv, dkp, rp):
    _check(lib().lester_set_gamsc1_bc(*map(_p, (sc1, gamsc1, gamlam, diu, djv, dkp, rp))))


def set_sc1(u, v, w, p, sc1, rho, gamsc1, gamlam, hsc1, metrics: dict, dkp, dkw):
    m = [_p(metrics[n]) for n in W_ROLES[:13]]
    _check(lib().lester_set_sc1(*map(_p, (u, v, w, p, sc1, rho, gamsc1, gamlam, hsc1)), *m,
                                _p(dkp), _p(dkw), None, None))


def set_sc1_bc(f):
    _check(lib().lester_set_sc1_bc(_p(f)))


def set_sc1var(u, v, w, sc1, rho, sc1var, sc1dis, dip, djp, dkp, dkw, rp):
    _check(lib().lester_set_sc1var(*map(_p, (u, v, w, sc1, rho, sc1var, sc1dis, dip, djp, dkp, dkw,
                                             rp)), None, None))


# ------------------------------------- convective outflow / fixed inflow
def conv_exitbc(task, iva, rho, rhonp1, u, v, w, u_int, v_int, w_int, hu, hv, hw, metrics: dict, dkp,
                dkw):
    """code/conv_exitbc.F:21 (metrics: the 2-D metric dict)."""
    m = metrics
    _check(lib().lester_conv_exitbc(_i(task), _i(iva), _p(rho), _p(rhonp1), _p(u), _p(v), _p(w),
                                    _p(u_int), _p(v_int), _p(w_int), _p(hu), _p(hv), _p(hw),
                                    *[_p(m[n]) for n in ("dip", "diu", "dix", "djp", "djv", "djx", "rdiv",
                                                         "rdju", "didjp", "rp", "ru", "rv")],
                                    _p(dkp), _p(dkw), _p(m["rdidjp"])))


def mass_change(rho, rhonp1, rdidjp, dkw) -> float:
    out = C.c_double()
    _check(lib().lester_mass_change(_p(rho), _p(rhonp1), C.byref(out), _p(rdidjp), _p(dkw)))
    return out.value


def gpu_set_inlet(inlet, uprof=None, vprof=None, seed: int = 0) -> None:
    """Inlet blocks (four 1-based block numbers, 0 = none) and the u, v
    inflow profiles (equal-length float64 arrays)."""
    ib = (C.c_int * 4)(*[int(b) for b in inlet])
    n = 0 if uprof is None else len(uprof)
    _check(lib().lester_gpu_set_inlet(ib, _p(uprof), _p(vprof), n, C.c_ulonglong(seed)))


def fixed_inlet(u_int, v_int, w_int, u, v, w, sc1, rho, iseed, uprof, vprof, step):
    """code/fixed_inlet.F:5 (the arguments it reads; the rest are passed as NULL)."""
    _check(lib().lester_fixed_inlet(None, None, None, _p(u_int), _p(v_int), _p(w_int), _p(u), _p(v), _p(w),
                                    None, _p(sc1), _p(rho), None, _i(iseed), None, _p(uprof), _p(vprof),
                                    None, None, None, None, None, None, None, None, None, None, _i(step)))


def recycling(u_int, v_int, w_int, u, v, w, sc1, rho, prof, means, step, inblock):
    """mas-recyc/recycling.F:5: prof = (uprof, vprof, wprof, uuprof, vvprof,
    wwprof), means = (umean, vmean, wmean, uumean, vvmean, wwmean)."""
    _check(lib().lester_recycling(None, None, None, _p(u_int), _p(v_int), _p(w_int), _p(u), _p(v), _p(w), None,
                                  _p(sc1), _p(rho), None, _i(0), None, *[_p(a) for a in prof],
                                  *[_p(a) for a in means], _i(step), _i(inblock)))


STAT_NAMES = "um vm wm pm rhom ruv rvw rwu ruu rvv rww rrh fm rff sc1varm T_m".split()


def statistics(u, v, w, p, rho, sc1, sc1var, gam, outs: dict, no_sam: int):
    """code/statistics.F:1 (the averaging): outs maps STAT_NAMES to 2-D
    arrays (level-1 metric layout), updated in place; no_sam the sample
    count including this one."""
    _check(lib().lester_gpu_set_stat_samples(int(no_sam)))
    o = outs
    _check(lib().lester_statistics(_p(u), _p(v), _p(w), _p(p), _p(rho), _p(o["um"]), _p(o["vm"]), _p(o["wm"]),
                                   _p(o["pm"]), _p(o["rhom"]), _p(o["ruv"]), _p(o["rvw"]), _p(o["rwu"]),
                                   _p(o["ruu"]), _p(o["rvv"]), _p(o["rww"]), _p(o["rrh"]), _p(gam), None,
                                   _p(sc1), _p(o["fm"]), _p(o["rff"]), _p(sc1var), None, _p(o["sc1varm"]), None,
                                   None, _p(o["T_m"]), None, None, None, None, None, None, None, None, _i(0)))
