"""Parity on the benchmarked configurations, scaled to sizes the oracle
finishes in seconds, through the C ABI (lester_step).

1. The headline path -- variable-density temporal mixing layer (density
   ratio 2 through the mixing law), tanh-stretched slip walls (beta 2),
   WALE Cw 0.5, the mixed solver to 1e-8 with FP32 physics, steps 2.. replayed
   from the whole-step graph -- at 64 x 48 x 32 cells with the headline's
   cell size, 5 steps.  Its FP64 reference is the oracle's step (code/step.F
   order) with the pressure source made compatible (interior mean removed,
   the part of a singular system any p can match, as the fast solvers do)
   and lmg_solve run to tolf 1e-14.  The per-field relative L2 error of the
   mixed path, and of the FP64 fast path beside it, is stated below and
   asserted.
2. The reference's own CPU-runnable case: the 64^3 plane channel, 4
   multigrid levels, Smagorinsky Cs 0.1, 10 steps at dt from CFL 0.3 --
   the reference solver mode against orc_step at 1e-10, and the fast
   solvers against a converged oracle at 1e-8.
"""
import numpy as np
import pytest

from fortranutils_gb300 import grid
from fortranutils_gb300 import lester as L
from fortranutils_gb300 import state as S

import oracle_lib as O

pytestmark = pytest.mark.gpu

FIELDS6 = ("u", "v", "w", "p", "sc1", "rho")


def rel(a, b):
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


def oracle_state(case, orc, init):
    x, y, z = case.coordinates()
    met, dkp, dkw = orc.comp_metric(x, y, z)
    m = {n: np.ascontiguousarray(met[i]) for i, n in enumerate(L.METRIC_NAMES)}
    s = S.new_state(case, m, dkp, dkw)
    init(s)
    # ghosts of the initial fields as lester_step's callers set them
    for n in ("u", "v", "w", "sc1", "rho", "rhonp1", "rhonm1"):
        orc.swap_sc(1, s[n], 2)
    return s


def run_oracle(orc, ctrl, s, nstep, mg):
    r = s.to("numpy")
    k = O.phys_from_ctrl(ctrl)
    for it in range(1, nstep + 1):
        orc.step(mg, k, it, it + 1, r)
    return r


def run_gpu(case, ctrl, s, nstep):
    g = s.to("torch")
    L.gpu_init(case.geom(), ctrl)
    try:
        rcs = [S.step(g, it) for it in range(1, nstep + 1)]
        info = L.gpu_step_graph_info()
        info["forms"] = L.gpu_solver_forms()
        L.gpu_sync()
        return g.to("numpy"), rcs, info
    finally:
        L.gpu_finalize()


# ---------------------------------------------------------------- headline
# The headline workload (256x192x128 on 30 x 30 x 15) at a quarter of the
# cells per axis on a quarter of the domain: the same cell sizes.
MIX_SHAPE, MIX_DOMAIN, MIX_STEPS = (64, 48, 32), (7.5, 7.5, 3.75), 5
MIX_CTRL = dict(dtime=0.01, model=2, csles=0.5, rholo=1.0, rhohi=2.0, rtol=1e-8, max_outer=200, exact=0,
                krylov=2)
# Per-field relative L2 after 5 steps against the compatible converged FP64
# oracle, measured on a GB300 (mixed + FP32 physics: u 4.8e-7, v 1.5e-5,
# w 1.4e-5, p 1.1e-5, sc1 9.7e-8, rho 7.7e-8; FP64 fast path: u 6.1e-11,
# v 5.1e-9, w 1.6e-9, p 5.6e-9, sc1 6.9e-11, rho 5.3e-11)
MIXED_TOL = {"u": 1e-6, "v": 2e-5, "w": 2e-5, "p": 2e-5, "sc1": 3e-7, "rho": 3e-7}
FP64_TOL = {"u": 3e-10, "v": 4e-8, "w": 1e-8, "p": 4e-8, "sc1": 1e-10, "rho": 1e-10}


def mixing_case():
    return grid.box_case(*MIX_SHAPE, lx=MIX_DOMAIN[0], ly=MIX_DOMAIN[1], lz=MIX_DOMAIN[2],
                         ybc=L.BCT_ZERO_GRAD, beta=2.0)


def test_headline_mixed_path_per_field_error(gpulib):
    case = mixing_case()
    orc = O.Oracle(case)
    ctrl = L.default_ctrl(psolve=L.PSOLVE_MIXED, phys32=1, **MIX_CTRL)
    s = oracle_state(case, orc, lambda st: S.init_mixing_layer(st, seed=2, sigma=0.02, rholo=1.0,
                                                                 rhohi=2.0))
    ref = run_oracle(orc, ctrl, s, MIX_STEPS, O.mgctrl(nummgits=500, tolf=1e-14, compat=1))
    fp64, rc64, _ = run_gpu(case, L.default_ctrl(psolve=L.PSOLVE_FP64, **MIX_CTRL), s, MIX_STEPS)
    launched, rcl, _ = run_gpu(case, ctrl, s, MIX_STEPS)
    ctrl.step_graph = 1
    replayed, rcg, info = run_gpu(case, ctrl, s, MIX_STEPS)
    assert rc64 == rcl == rcg == [0] * MIX_STEPS
    assert not info["failed"] and info["replays"] == MIX_STEPS - 1, info
    # the headline's solver forms: FP32 couplings and the double-float
    # residual from separable factors, the bottom level solved exactly
    f = info["forms"]
    assert f["mf32"] and f["df_separable"] and f["df_diag_sum"] and f["direct32"], f
    for n in S.STATE:
        assert np.array_equal(replayed[n], launched[n]), n
    e_mx = {n: rel(replayed[n], ref[n]) for n in FIELDS6}
    e_64 = {n: rel(fp64[n], ref[n]) for n in FIELDS6}
    print("\nmixing layer 64x48x32, 5 steps, rel L2 vs compatible converged FP64 oracle: mixed+FP32 physics "
          + ", ".join(f"{n} {e:.2e}" for n, e in e_mx.items()) + "; FP64 fast path "
          + ", ".join(f"{n} {e:.2e}" for n, e in e_64.items()))
    for n in FIELDS6:
        assert e_mx[n] <= MIXED_TOL[n], ("mixed", n, e_mx[n])
        assert e_64[n] <= FP64_TOL[n], ("fp64", n, e_64[n])
    assert rel(replayed["u"], s["u"]) > 1e-4  # the flow moved


# ------------------------------------------------------------ 64^3 channel
CH_STEPS = 10


def channel_setup():
    case = grid.box_case(64, 64, 64, ybc=L.BCT_WALL, nummgl=4)
    orc = O.Oracle(case)
    s = oracle_state(case, orc, lambda st: S.init_channel(st, seed=1, sigma=0.05))
    # dt from CFL 0.3 and diffusion number 0.2 of the initial field, fixed
    cmax, dmax, visc = 0.0, 0.0, 1.0 / 2800.0
    b = case.blocks[0]
    dx, dy, dz = (np.diff(a[1:n]).min() for a, n in ((b.x, b.n[0]), (b.y, b.n[1]), (b.z, b.n[2])))
    u, v, w = (case.block_view(s[n], 0)[1:-1, 1:-1, 1:-1] for n in "uvw")
    cmax = float((np.abs(u) / dx + np.abs(v) / dy + np.abs(w) / dz).max())
    dmax = visc * (1.0 / dx ** 2 + 1.0 / dy ** 2 + 1.0 / dz ** 2)
    dt = min(0.3 / cmax, 0.2 / dmax)
    return case, orc, s, dict(dtime=dt, model=1, csles=0.1, rholo=1.0, rhohi=1.0, visc=visc)


def test_channel64_reference_solver(gpulib):
    """The reference solver mode (lexicographic SOR V-cycles, the
    reference's stop rule) on the 64^3 channel with 4 levels: every carried
    field within 1e-10 of orc_step after 10 steps."""
    case, orc, s, kw = channel_setup()
    ctrl = L.default_ctrl(psolve=L.PSOLVE_REFERENCE, exact=1, **kw)
    ref = run_oracle(orc, ctrl, s, CH_STEPS, O.mgctrl_from_ctrl(ctrl))
    got, rcs, _ = run_gpu(case, ctrl, s, CH_STEPS)
    assert rcs == [0] * CH_STEPS
    bad = {n: rel(got[n], ref[n]) for n in S.STATE if rel(got[n], ref[n]) > 1e-10}
    assert not bad, bad
    assert rel(got["u"], s["u"]) > 1e-4


@pytest.mark.parametrize("psolve", [L.PSOLVE_FP64, L.PSOLVE_MIXED])
def test_channel64_fast_solvers(psolve, gpulib):
    """The fast solvers (to 1e-10) on the 64^3 channel against an oracle
    whose V-cycles run to tolf 1e-14: u, v, w within 1e-8 after 10 steps,
    p within 1e-6 (measured: u 9.2e-13, v 2.5e-12, w 1.4e-12, p 8.1e-11);
    with FP32 physics (the mixed path: u 9.4e-8, v 5.9e-7, w 4.4e-7,
    p 1.1e-5) within the FP32 bounds."""
    case, orc, s, kw = channel_setup()
    ctrl = L.default_ctrl(psolve=psolve, rtol=1e-10, exact=0, **kw)
    ref = run_oracle(orc, ctrl, s, CH_STEPS, O.mgctrl(nummgits=400, tolf=1e-14))
    got, rcs, _ = run_gpu(case, ctrl, s, CH_STEPS)
    assert rcs == [0] * CH_STEPS
    errs = {n: rel(got[n], ref[n]) for n in ("u", "v", "w", "p")}
    print(f"\nchannel64 psolve {psolve}, 10 steps: " + ", ".join(f"{n} {e:.2e}" for n, e in errs.items()))
    for n in ("u", "v", "w"):
        assert errs[n] <= 1e-8, (n, errs[n])
    assert errs["p"] <= 1e-6
    if psolve == L.PSOLVE_MIXED:
        ctrl.phys32 = 1
        got32, rcs32, _ = run_gpu(case, ctrl, s, CH_STEPS)
        assert rcs32 == [0] * CH_STEPS
        e32 = {n: rel(got32[n], ref[n]) for n in ("u", "v", "w", "p")}
        print("  with FP32 physics: " + ", ".join(f"{n} {e:.2e}" for n, e in e32.items()))
        for n, tol in (("u", 5e-7), ("v", 3e-6), ("w", 3e-6), ("p", 5e-5)):
            assert e32[n] <= tol, (n, e32[n])
