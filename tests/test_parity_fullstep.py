"""GPU parity of whole time steps (lester_step, the ivar loop of
code/step.F:214-454) against the oracle's orc_step, through the C ABI.

Bar: relative L2 <= 1e-10 on every field the step carries to the next one
after several steps with the reference solver (the per-routine tests hold
the routines bitwise; the step adds the 1e-13 log/pow differences of the
wall functions and eddy viscosity, which the pressure solve spreads).
The fast solvers are checked against a converged oracle solve.
"""
import numpy as np
import pytest

from fortranutils_gb300 import lester as L
from fortranutils_gb300 import state as S

import cases
import oracle_lib as O

pytestmark = pytest.mark.gpu

NSTEP = 3
RTOL_STEP = 1e-10

SETUPS = {
    # channel: walls in y, Smagorinsky
    "box_wall": dict(init="channel", model=1),
    # mixing layer: slip walls, stretched y, WALE, variable density
    "box_slip_stretched": dict(init="mixing", model=2, rholo=1.0, rhohi=2.0),
    # two blocks joined by interfaces, no eddy-viscosity model
    "two_block": dict(init="channel", model=0),
}


def make(name, **ctrl_kw):
    cfg = dict(SETUPS[name])
    init = cfg.pop("init")
    st = cases.Setup(name)
    cfg.update(ctrl_kw)
    ctrl = L.default_ctrl(dtime=2e-3, **cfg)
    s = S.new_state(st.case, st.m, st.dkp, st.dkw)
    if init == "channel":
        S.init_channel(s, seed=5)
    else:
        S.init_mixing_layer(s, seed=6, rholo=ctrl.rholo, rhohi=ctrl.rhohi)
    return st, ctrl, s


def rel(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)


def oracle_steps(st, ctrl, s, nstep, mg=None):
    ref = s.to("numpy")
    mg = mg or O.mgctrl_from_ctrl(ctrl)
    k = O.phys_from_ctrl(ctrl)
    for it in range(1, nstep + 1):
        st.orc.step(mg, k, it, it + 1, ref)
    return ref


def gpu_steps(st, ctrl, s, nstep, kind="torch"):
    g = s.to(kind)
    L.gpu_init(st.case.geom(), ctrl)
    try:
        rcs = [S.step(g, it) for it in range(1, nstep + 1)]
        L.gpu_sync()
        return g.to("numpy"), rcs
    finally:
        L.gpu_finalize()


@pytest.mark.parametrize("exact", [1, 0])
@pytest.mark.parametrize("name", list(SETUPS))
def test_steps_reference_solver(name, exact, gpulib):
    """Both builds of the FP64 physics kernels against the oracle."""
    st, ctrl, s = make(name, exact=exact)
    ref = oracle_steps(st, ctrl, s, NSTEP)
    got, rcs = gpu_steps(st, ctrl, s, NSTEP)
    assert rcs == [0] * NSTEP
    bad = {n: rel(got[n], ref[n]) for n in S.STATE if rel(got[n], ref[n]) > RTOL_STEP}
    assert not bad, bad
    # the velocities moved: the step did work
    assert rel(got["u"], s["u"]) > 1e-6


def host_state_equal(hst, dev, st):
    """The fields lester_step returns to host arrays equal the device run's:
    the carried state, p on level 1 (the coarser levels are solver work)."""
    n3 = st.case.n3_sg
    for n in S.STATE:
        a, b = (hst[n][:n3], dev[n][:n3]) if n == "p" else (hst[n], dev[n])
        np.testing.assert_array_equal(a, b, err_msg=n)


@pytest.mark.parametrize("name,kw", [("box_wall", {}), ("box_slip_stretched", {"model": 1})])
def test_steps_host_arrays_match_device(name, kw, gpulib):
    """Host (numpy, pageable) fields through the same entry point: copied
    in and out once per call, same numbers as device-resident fields.  The
    slip-wall Smagorinsky case reads vd_damping where no wall writes it."""
    st, ctrl, s = make(name, **kw)
    dev, _ = gpu_steps(st, ctrl, s, 2, "torch")
    hst, _ = gpu_steps(st, ctrl, s, 2, "numpy")
    host_state_equal(hst, dev, st)


@pytest.mark.parametrize("graph", [0, 1])
def test_host_arrays_fast_path(graph, gpulib):
    """The benchmarked path (mixed solver, FP32 physics) with host arrays,
    steps 2.. replayed from the whole-step graph or launched: the state the
    host gets back equals the device-resident run bit for bit, and the
    pressure coefficients cross to the device once after the first step."""
    st, ctrl, s = make("box_slip_stretched", psolve=L.PSOLVE_MIXED, rtol=1e-9, exact=0, phys32=1,
                       step_graph=graph)
    dev, rd = gpu_steps(st, ctrl, s, 4, "torch")
    g = s.to("pinned")
    L.gpu_init(st.case.geom(), ctrl)
    try:
        rh = [S.step(g, 1), S.step(g, 2)]
        b0 = L.gpu_xfer_bytes()
        rh += [S.step(g, it) for it in (3, 4)]
        b1 = L.gpu_xfer_bytes()
        info = L.gpu_step_graph_info()
        hst = g.to("numpy")
    finally:
        L.gpu_finalize()
    assert rh == rd
    if graph:
        assert info["replays"] == 3 and not info["failed"], info
    host_state_equal(hst, dev, st)
    # per step in: the carried state, p on level 1, metrics and wall
    # arrays; no coefficient or work array
    carried = ("u v w sc1 rho hn_u hn_v hn_w hn_sc1 gam gamsc1 sc1var sc1dis vd_damping "
               "temperature").split()
    want_in = (sum(g[n].size for n in carried + S.TW) + st.case.n3_sg + g["dkp"].size + g["dkw"].size
               + sum(a.size for a in g["metric"].values()))
    assert (b1[0] - b0[0]) == 2 * 8 * want_in, (b1[0] - b0[0], want_in)


@pytest.mark.parametrize("psolve", [L.PSOLVE_FP64, L.PSOLVE_MIXED])
@pytest.mark.parametrize("name", ["box_wall", "box_slip_stretched"])
def test_steps_fast_solver(name, psolve, gpulib):
    """Fast solvers to rtol 1e-10 against an oracle run whose V-cycles
    continue to tolf (a converged reference solve)."""
    # constant density: a compatible pressure equation, so the reference's
    # SOR converges to the same solution the fast solvers find
    st, ctrl, s = make(name, psolve=psolve, rtol=1e-10, rholo=1.0, rhohi=1.0)
    ref = oracle_steps(st, ctrl, s, 2, O.mgctrl(nummgits=400, tolf=1e-14))
    got, rcs = gpu_steps(st, ctrl, s, 2)
    assert rcs == [0, 0]
    for n in ("u", "v", "w", "sc1", "rho"):
        assert rel(got[n], ref[n]) < 1e-8, (n, rel(got[n], ref[n]))
    assert rel(got["p"], ref["p"]) < 1e-6


def test_step_rejects_missing_field(gpulib):
    st, ctrl, s = make("box_wall")
    g = s.to("torch")
    del g["p"]
    L.gpu_init(st.case.geom(), ctrl)
    try:
        with pytest.raises(L.LesterError):
            S.step(g, 1)
    finally:
        L.gpu_finalize()


@pytest.mark.parametrize("psolve", [L.PSOLVE_FP64, L.PSOLVE_MIXED])
def test_variable_density_fast_solver_converges(psolve, gpulib):
    """Density ratio 2 between slip walls: the source has a net part no
    pressure can balance; the fast solvers converge on the rest."""
    st, ctrl, s = make("box_slip_stretched", psolve=psolve, rtol=1e-8)
    got, rcs = gpu_steps(st, ctrl, s, 3)
    assert rcs == [0, 0, 0]
    for n in S.STATE:
        assert np.all(np.isfinite(got[n])), n


GRAPH_VARIANTS = {
    "converged": dict(rtol=1e-9, max_outer=60),
    # every solve stops at max_outer: the step carries on (NOT_CONVERGED)
    "max_outer": dict(rtol=1e-12, max_outer=2),
    # a poor smoother: defect-correction cycles stall, the auto mode hands
    # the solve to flexible CG (on the host, after the replayed part)
    "stall": dict(rtol=1e-9, max_outer=60, rb_sweeps=1, rb_omega=1.95),
}


GRAPH_CASES = [(v, k) for v in GRAPH_VARIANTS for k in (0, 1, 2) if not (v == "stall" and k == 0)]
# the benchmarked path: FP32 physics (les_f32) replayed from the graph
GRAPH_F32 = dict(exact=0, phys32=1)


# (the stall variant diverges with plain defect correction, krylov 0)
@pytest.mark.parametrize("physics", ["fp64", "f32"])
@pytest.mark.parametrize("variant,krylov", GRAPH_CASES)
@pytest.mark.parametrize("psolve", [L.PSOLVE_FP64, L.PSOLVE_MIXED])
@pytest.mark.parametrize("name", list(SETUPS))
def test_step_graph_replays_bitwise(name, psolve, krylov, variant, physics, gpulib):
    """ctrl.step_graph: steps 2..5 replayed from one captured graph (the
    solve's cycle loop a device-side WHILE node, the rest of the step behind
    an IF node) give the fields of the steps launched call by call, bit for
    bit, and the same return codes."""
    if physics == "f32" and (psolve != L.PSOLVE_MIXED or variant == "max_outer"):
        pytest.skip("FP32 physics: with the mixed solver, converged and stalling solves")
    n = 5
    extra = GRAPH_F32 if physics == "f32" else {}
    st, ctrl, s = make(name, psolve=psolve, krylov=krylov, **GRAPH_VARIANTS[variant], **extra)
    plain, rc0 = gpu_steps(st, ctrl, s, n)
    ctrl.step_graph = 1
    g = s.to("torch")
    L.gpu_init(st.case.geom(), ctrl)
    try:
        rcs = [S.step(g, it) for it in range(1, n + 1)]
        info = L.gpu_step_graph_info()
        L.gpu_sync()
        got = g.to("numpy")
    finally:
        L.gpu_finalize()
    assert rcs == rc0
    if variant == "max_outer":
        assert rcs[1:] == [-7] * (n - 1)  # LES_ERR_NOT_CONVERGED
    assert not info["failed"], info["why"]
    assert info["replays"] == n - 1
    if variant == "stall" and krylov == 2:  # the handover to the host loop ran
        assert info["handovers"] > 0
    for f in S.STATE:
        assert np.all(np.isfinite(plain[f])), f
        assert np.array_equal(got[f], plain[f]), f


# ctrl.phys32: the mixed path with FP32 arithmetic in the predictors, the
# scalar transport and the eddy viscosity (FP64 fields, FP64 fine-grid
# residual and sums).  Its error against the FP64 oracle, per field, after
# two steps at constant density (so that the reference's SOR converges to
# the solution the fast solvers find), relative L2:
# (measured on the three cases: u 3.3e-8 to 3.8e-8, v 2.3e-7 to 3.6e-7,
# w 1.8e-7 to 2.1e-7, sc1 3.1e-8, p 4.0e-7 to 1.0e-6)
PHYS32_TOL = {"u": 2e-7, "v": 2e-6, "w": 2e-6, "sc1": 2e-7, "rho": 1e-12, "p": 1e-5}


@pytest.mark.parametrize("name", list(SETUPS))
def test_phys32_error_per_field(name, gpulib):
    """The FP32-arithmetic physics build with the mixed solver against a
    converged FP64 oracle: every field within its stated tolerance, and
    the FP64 physics build an order of magnitude or more closer."""
    st, ctrl, s = make(name, psolve=L.PSOLVE_MIXED, rtol=1e-10, rholo=1.0, rhohi=1.0, exact=0)
    ref = oracle_steps(st, ctrl, s, 2, O.mgctrl(nummgits=400, tolf=1e-14))
    fp64, _ = gpu_steps(st, ctrl, s, 2)
    ctrl.phys32 = 1
    got, rcs = gpu_steps(st, ctrl, s, 2)
    assert rcs == [0, 0]
    errs = {n: rel(got[n], ref[n]) for n in PHYS32_TOL}
    errs64 = {n: rel(fp64[n], ref[n]) for n in PHYS32_TOL}
    print(f"\n{name} phys32 rel L2: " + ", ".join(f"{n} {e:.1e}" for n, e in errs.items()) +
          "; FP64 physics: " + ", ".join(f"{n} {e:.1e}" for n, e in errs64.items()))
    for n, tol in PHYS32_TOL.items():
        assert errs[n] <= tol, (n, errs[n], tol)
    assert rel(got["u"], s["u"]) > 1e-6  # the step did work


def test_step_graph_recaptures_on_new_fields_and_controls(gpulib):
    """The graph is captured per field set and controls: moving the state to
    new device arrays, then changing dtime, gives new captures, and the run
    stays bit for bit the launched one."""
    def run(graph):
        st, ctrl, s = make("box_wall", psolve=L.PSOLVE_MIXED, rtol=1e-9, exact=0, phys32=1)
        ctrl.step_graph = graph
        g = s.to("torch")
        L.gpu_init(st.case.geom(), ctrl)
        try:
            for it in (1, 2, 3):
                assert S.step(g, it) == 0
            g = g.to("numpy").to("torch")  # the same state in new arrays
            for it in (4, 5):
                assert S.step(g, it) == 0
            ctrl.dtime = 1.5e-3
            L.gpu_set_ctrl(ctrl)
            for it in (6, 7):
                assert S.step(g, it) == 0
            info = L.gpu_step_graph_info()
            L.gpu_sync()
            return g.to("numpy"), info
        finally:
            L.gpu_finalize()

    plain, _ = run(0)
    got, info = run(1)
    # step 4, the first on the new arrays, runs as launched (it converts the
    # new coefficient arrays for the fast solver); captures at 2, 5 and 6
    assert not info["failed"] and info["replays"] == 5, info
    for f in S.STATE:
        assert np.array_equal(got[f], plain[f]), f


def test_step_log_lines(tmp_path, gpulib):
    """lester_gpu_step_log: one JSON line per step with the solve's cycles,
    residual norms, the replay flag and the bytes copied; closing the log
    stops the lines."""
    import json
    st, ctrl, s = make("box_wall", psolve=L.PSOLVE_MIXED, rtol=1e-9, exact=0, phys32=1, step_graph=1)
    log = tmp_path / "steps.jsonl"
    g = s.to("pinned")
    L.gpu_init(st.case.geom(), ctrl)
    try:
        L.gpu_step_log(log)
        rcs = [S.step(g, it) for it in (1, 2, 3)]
        L.gpu_step_log(None)
        S.step(g, 4)
    finally:
        L.gpu_finalize()
    lines = [json.loads(x) for x in log.read_text().splitlines()]
    assert [d["istep"] for d in lines] == [1, 2, 3] and [d["rc"] for d in lines] == rcs == [0, 0, 0]
    assert [d["graph"] for d in lines] == [False, True, True]
    for d in lines:
        assert d["vcycles"] > 0 and 0 < d["relres"] <= 1e-9 and d["ms"] > 0
        assert d["resid_rms"] == pytest.approx(d["relres"] * d["rhs_rms"], rel=1e-6)
        assert d["h2d_bytes"] > 0 and d["d2h_bytes"] > 0


@pytest.mark.parametrize("graph", [0, 1])
def test_rb_tile_smoother(graph, gpulib):
    """ctrl.rb_tile: the mixed solver's level-1 red-black sweeps through
    shared-memory tiles (one launch per sweep, the colour-0 halo recomputed)
    on the one-block periodic/slip case: the smoother is in use and three
    steps agree with the per-colour sweeps to the solver's tolerance (the
    two kernels contract their sums differently)."""
    # mg_tail 0: per-level launches (the single-CTA tail would take every
    # level of this small case)
    st, ctrl, s = make("box_slip_stretched", psolve=L.PSOLVE_MIXED, rtol=1e-10, exact=0, phys32=1,
                       step_graph=graph, autotune=0, mg_tail=0)
    ref, rc0 = gpu_steps(st, ctrl, s, 3)
    ctrl.rb_tile = 1
    g = s.to("torch")
    L.gpu_init(st.case.geom(), ctrl)
    try:
        rcs = [S.step(g, it) for it in (1, 2, 3)]
        mask = L.gpu_rb_tiles()
        L.gpu_sync()
        got = g.to("numpy")
    finally:
        L.gpu_finalize()
    assert rcs == rc0 == [0, 0, 0]
    assert mask & 2, mask  # level 1 smoothed by the tiles
    for n in ("u", "v", "w", "p", "sc1"):
        assert rel(got[n], ref[n]) <= 1e-7, (n, rel(got[n], ref[n]))


def test_p_guess_extrapolation(gpulib):
    """ctrl.p_guess: the fast solves starting from 2 p(n) - p(n-1) (1) or
    from p(n) (0, the default) reach the same fields to the solver's
    tolerance."""
    st, ctrl, s = make("box_slip_stretched", psolve=L.PSOLVE_MIXED, rtol=1e-10, exact=0, phys32=1)
    res = {}
    for guess in (1, 0):
        ctrl.p_guess = guess
        g = s.to("torch")
        L.gpu_init(st.case.geom(), ctrl)
        try:
            cyc = 0
            for it in range(1, 7):
                assert S.step(g, it) == 0
                cyc += L.gpu_solve_stats()["cycles"]
            L.gpu_sync()
            res[guess] = (g.to("numpy"), cyc)
        finally:
            L.gpu_finalize()
    (a, ca), (b, cb) = res[1], res[0]
    # a residual of 1e-10 bounds p's error only up to the operator's
    # condition number: p within 1e-5, as the FP32 physics' stated bound
    for n, tol in (("u", 1e-7), ("v", 1e-7), ("w", 1e-7), ("sc1", 1e-7), ("p", 1e-5)):
        assert rel(a[n], b[n]) <= tol, (n, rel(a[n], b[n]))
    print(f"\nV-cycles over 6 steps: extrapolated start {ca}, previous p {cb}")
