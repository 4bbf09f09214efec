"""Arrays of one LES time step and their initial values.

``State`` holds every field ``lester_step`` reads or writes (the arena
slices of code/step.F), as numpy arrays (host) or torch CUDA tensors
(device), in the reference's layout.  Initial fields are seeded synthetic
data; no reference input deck is read.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lester as L

FIELDS3 = ("u v w sc1 rho rhonp1 rhonm1 u_int v_int w_int hn_u hn_v hn_w hn_sc1 gam gamsc1 gamlam "
           "sc1var sc1dis vd_damping temperature drhonp1dt srhot srhoux").split()
FIELDSM = "p s res ap aw ae as an al ar".split()
TW = ("tw_sfi tw_nfi tw_lfi tw_rfi tw_wfj tw_efj tw_lfj tw_rfj tw_wfk tw_efk tw_sfk "
      "tw_nfk").split()
# the state a time step carries to the next one (scratch excluded)
STATE = ("u v w p sc1 rho rhonp1 rhonm1 hn_u hn_v hn_w hn_sc1 gam gamsc1 gamlam sc1var sc1dis "
         "vd_damping temperature").split() + TW


class Fields(C.Structure):
    """include/lester_gpu.h lester_fields"""
    _fields_ = ([(n, C.c_void_p) for n in FIELDS3] + [(n, C.c_void_p) for n in FIELDSM] +
                [("metric", C.c_void_p * 35), ("dkp", C.c_void_p), ("dkw", C.c_void_p),
                 ("tw", C.c_void_p * 12)])


def tw_sizes(case) -> dict:
    lev = case.levels[0]
    ki = sum(c * a for (a, b, c) in lev)
    jk = sum(b * c for (a, b, c) in lev)
    ij = sum(a * b for (a, b, c) in lev)
    return {"tw_sfi": ki, "tw_nfi": ki, "tw_lfi": ij, "tw_rfi": ij, "tw_wfj": jk, "tw_efj": jk,
            "tw_lfj": ij, "tw_rfj": ij, "tw_wfk": jk, "tw_efk": jk, "tw_sfk": ki, "tw_nfk": ki}


class State(dict):
    """name -> array; also ``metric`` (dict of 35) and ``dkp``, ``dkw``."""

    def __init__(self, case):
        super().__init__()
        self.case = case

    def fields(self) -> Fields:
        """ctypes view of the arrays (kept alive by this State)."""
        f = Fields()
        for n in FIELDS3 + FIELDSM:
            a = self.get(n)
            setattr(f, n, None if a is None else L._p(a).value)
        for q, n in enumerate(L.METRIC_NAMES):
            f.metric[q] = L._p(self["metric"][n]).value
        f.dkp = L._p(self["dkp"]).value
        f.dkw = L._p(self["dkw"]).value
        for q, n in enumerate(TW):
            f.tw[q] = L._p(self[n]).value
        return f

    def to(self, kind: str) -> "State":
        """Copy to 'numpy', 'torch' (CUDA) or 'pinned' (torch pinned host, numpy view)."""
        out = State(self.case)
        conv = _converter(kind)
        for k, v in self.items():
            if k == "metric":
                out[k] = {n: conv(a) for n, a in v.items()}
            else:
                out[k] = conv(v)
        return out


def _converter(kind):
    if kind == "numpy":
        def f(a):
            return np.ascontiguousarray(a.cpu().numpy() if hasattr(a, "cpu") else a).copy()
        return f
    import torch
    if kind == "torch":
        def f(a):
            return (a if hasattr(a, "cuda") and not isinstance(a, np.ndarray) else
                    torch.from_numpy(np.ascontiguousarray(a))).cuda().clone()
        return f
    if kind == "pinned":
        def f(a):
            t = a.cpu() if hasattr(a, "cpu") and not isinstance(a, np.ndarray) else torch.from_numpy(a)
            return t.contiguous().pin_memory().numpy()
        return f
    raise ValueError(kind)


def new_state(case, metrics: dict, dkp, dkw) -> State:
    """Zero fields (numpy) for ``case`` with the given comp_metric output."""
    s = State(case)
    for n in FIELDS3:
        s[n] = np.zeros(case.n3_sg)
    for n in FIELDSM:
        s[n] = np.zeros(case.n3_mg)
    for n, sz in tw_sizes(case).items():
        s[n] = np.zeros(sz)
    s["metric"] = {n: np.ascontiguousarray(metrics[n]) for n in L.METRIC_NAMES}
    s["dkp"] = np.ascontiguousarray(dkp)
    s["dkw"] = np.ascontiguousarray(dkw)
    return s


def cell_centre_y(case, ib: int = 0) -> np.ndarray:
    """y at the cell centres j = 1..njp1 of block ib (ghosts by linear
    extrapolation); for a block with 2-D vertices (a deck), along its first
    interior i line."""
    b = case.blocks[ib]
    if b.xv is not None:
        yv = np.zeros(b.n[1] + 1)
        yv[1:b.n[1]] = 0.5 * (b.yv[:, 0] + b.yv[:, 1])
    else:
        yv = b.y.copy()
    yv[0] = 2 * yv[1] - yv[2]
    yv[-1] = 2 * yv[-2] - yv[-3]
    return 0.5 * (yv[:-1] + yv[1:])[: b.n[1]]


def _close_walls(s: State) -> None:
    """No flow through solid or slip y sides: v = 0 on the south face of the
    first interior cell and of the north ghost cell (the wall faces, which
    no routine of the step writes)."""
    c = s.case
    for ib, b in enumerate(c.blocks):
        v = c.block_view(s["v"], ib)
        if b.bc[2] in (L.BCT_WALL, L.BCT_ZERO_GRAD):
            v[:, 1, :] = 0.0
        if b.bc[3] in (L.BCT_WALL, L.BCT_ZERO_GRAD):
            v[:, -1, :] = 0.0


def init_channel(s: State, seed: int = 1, sigma: float = 0.05) -> State:
    """u = 1 - y^2 + N(0, sigma^2), v, w = N(0, sigma^2), rho = 1."""
    rng = np.random.default_rng(seed)
    c = s.case
    for ib, b in enumerate(c.blocks):
        nip1, njp1, nkp1 = b.n
        yc = cell_centre_y(c, ib)
        sh = (nkp1, njp1, nip1)
        c.block_view(s["u"], ib)[...] = (1.0 - yc ** 2)[None, :, None] + sigma * rng.standard_normal(sh)
        c.block_view(s["v"], ib)[...] = sigma * rng.standard_normal(sh)
        c.block_view(s["w"], ib)[...] = sigma * rng.standard_normal(sh)
    _close_walls(s)
    for n in ("rho", "rhonp1", "rhonm1"):
        s[n][:] = 1.0
    s["vd_damping"][:] = 1.0
    return s


def init_mixing_layer(s: State, seed: int = 2, sigma: float = 0.02, rholo: float = 1.0,
                      rhohi: float = 2.0) -> State:
    """u = 0.5 tanh(2y), scalar 0.5(1 + tanh(2y)), rho from the mixing law."""
    rng = np.random.default_rng(seed)
    c = s.case
    for ib, b in enumerate(c.blocks):
        nip1, njp1, nkp1 = b.n
        yc = cell_centre_y(c, ib)
        sh = (nkp1, njp1, nip1)
        c.block_view(s["u"], ib)[...] = 0.5 * np.tanh(2.0 * yc)[None, :, None] + sigma * rng.standard_normal(sh)
        c.block_view(s["v"], ib)[...] = sigma * rng.standard_normal(sh)
        c.block_view(s["w"], ib)[...] = sigma * rng.standard_normal(sh)
        c.block_view(s["sc1"], ib)[...] = np.broadcast_to(0.5 * (1.0 + np.tanh(2.0 * yc))[None, :, None], sh)
    _close_walls(s)
    f = s["sc1"]
    rho = 1.0 / (f / rhohi + (1.0 - f) / rholo)
    for n in ("rho", "rhonp1", "rhonm1"):
        s[n][:] = rho
    s["vd_damping"][:] = 1.0
    return s


def init_bl6(s: State, seed: int = 3, sigma: float = 0.03, delta: float = 0.5, rholo: float = 1.0,
             rhohi: float = 1.5, width: float = 0.0) -> State:
    """Boundary layer of grid.bl6_case: u = tanh(y / delta) + N(0, sigma^2),
    v, w = N(0, sigma^2); the scalar 0 below y = 2 (the lower row of blocks)
    and 1 above it, as a step (width 0) or 0.5 (1 + tanh((y - 2) / width)),
    rho from the mixing law.  (A step in density leaving through the
    convective outflow makes the reference scheme's first steps blow up at
    full resolution; the smooth form does not.)"""
    rng = np.random.default_rng(seed)
    c = s.case
    for ib, b in enumerate(c.blocks):
        nip1, njp1, nkp1 = b.n
        yc = 0.5 * (b.y[:-1] + b.y[1:])[:njp1]
        sh = (nkp1, njp1, nip1)
        c.block_view(s["u"], ib)[...] = np.tanh(np.maximum(yc, 0.0) / delta)[None, :, None] + \
            sigma * rng.standard_normal(sh)
        c.block_view(s["v"], ib)[...] = sigma * rng.standard_normal(sh)
        c.block_view(s["w"], ib)[...] = sigma * rng.standard_normal(sh)
        if width > 0.0:
            f = 0.5 * (1.0 + np.tanh((yc - 2.0) / width))
            c.block_view(s["sc1"], ib)[...] = np.broadcast_to(f[None, :, None], sh)
        else:
            c.block_view(s["sc1"], ib)[...] = 0.0 if ib < 3 else 1.0
    _close_walls(s)
    f = s["sc1"]
    rho = 1.0 / (f / rhohi + (1.0 - f) / rholo)
    for n in ("rho", "rhonp1", "rhonm1"):
        s[n][:] = rho
    s["vd_damping"][:] = 1.0
    return s


def step(state: State, istep: int) -> int:
    """lester_step on the state's arrays; returns the status (0, or
    LES_ERR_NOT_CONVERGED when a fast solver stopped short) and raises on
    any other error."""
    f = state.fields()
    rc = L.lib().lester_step(C.byref(f), L._i(istep))
    if rc not in (0, -7):
        L._check(rc)
    return rc


def _adj_cfg(nsteps, j_first, j_last, checkpoint):
    return L.AdjCfg(int(nsteps), int(j_first), int(j_last if j_last is not None else nsteps),
                    int(checkpoint if checkpoint is not None else nsteps))


def adjoint_run(state: State, nsteps: int, gfu, gfv, gfw, j_first: int = 1, j_last: int | None = None,
                checkpoint: int | None = None) -> float:
    """lester_adjoint_run: the objective J (mean wall shear stress over
    steps j_first..j_last of an nsteps run from ``state``, which is left
    unchanged) and its gradient with respect to the body force, written to
    the device tensors gfu, gfv, gfw."""
    f = state.fields()
    cfg = _adj_cfg(nsteps, j_first, j_last, checkpoint)
    J = C.c_double()
    L._check(L.lib().lester_adjoint_run(C.byref(cfg), C.byref(f), C.byref(J), L._p(gfu), L._p(gfv),
                                        L._p(gfw)))
    return J.value


def tangent_run(state: State, nsteps: int, dfu, dfv, dfw, j_first: int = 1, j_last: int | None = None):
    """lester_tangent_run: (J, dJ), dJ the derivative of J along the body
    force direction (dfu, dfv, dfw); ``state`` is left unchanged."""
    f = state.fields()
    cfg = _adj_cfg(nsteps, j_first, j_last, None)
    J, dJ = C.c_double(), C.c_double()
    L._check(L.lib().lester_tangent_run(C.byref(cfg), C.byref(f), L._p(dfu), L._p(dfv), L._p(dfw), C.byref(J),
                                        C.byref(dJ)))
    return J.value, dJ.value
