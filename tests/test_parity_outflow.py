"""GPU parity of the convective outflow and fixed inflow sides
(lester_conv_exitbc, lester_mass_change, lester_fixed_inlet and whole
steps through lester_step) against the oracle, on a two-block channel with
a BCT_FIXED inflow on block 1's west side and a BCT_CONVECTIVE outflow on
block 2's east side.

Bars: the inflow planes bitwise (the perturbation generator is the same
counter-based function on both sides); the exit planes and the mass change
relative 1e-12 (their side sums are tree reductions here, sequential sums
in the oracle); three whole steps relative L2 1e-10 per field.
"""
import numpy as np
import pytest

from fortranutils_gb300 import grid
from fortranutils_gb300 import lester as L
from fortranutils_gb300 import state as S

import cases
import oracle_lib as O

pytestmark = pytest.mark.gpu

INLET = [1, 0, 0, 0]
SEED = 12345


def setup():
    case = grid.inflow_case(12, 8, 8, 6)
    cases.CASES["inflow"] = lambda: case
    try:
        return cases.Setup("inflow", seed=3)
    finally:
        del cases.CASES["inflow"]


def profiles(case):
    nj = case.blocks[0].n[1] - 1
    n = case.blocks[0].n[1] + 3 * (nj - 1) + 8
    y = np.linspace(-1.0, 1.0, n)
    return np.ascontiguousarray(1.0 - y ** 2 + 0.1), np.ascontiguousarray(0.01 * y)


def state(st, seed):
    s = S.new_state(st.case, st.m, st.dkp, st.dkw)
    S.init_channel(s, seed=seed)
    rng = np.random.default_rng(seed + 1)
    s["rhonp1"][:] = 1.0 + 1e-4 * rng.random(s["rhonp1"].shape)
    for n in ("u", "v", "w"):
        s[n + "_int"][:] = s[n] + 0.01 * rng.standard_normal(s[n].shape)
    for n in ("hn_u", "hn_v", "hn_w"):
        s[n][:] = 0.1 * rng.standard_normal(s[n].shape)
    return s


def rel(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)


@pytest.fixture
def env(gpulib):
    st = setup()
    L.gpu_init(st.case.geom(), L.default_ctrl(dtime=2e-3))
    yield st
    L.gpu_finalize()


def test_mass_change(env):
    st = env
    s = state(st, 4)
    ref = st.orc.mass_change(2e-3, s["rho"], s["rhonp1"], st.m["rdidjp"], st.dkw)
    g = s.to("torch")
    got = L.mass_change(g["rho"], g["rhonp1"], g["metric"]["rdidjp"], g["dkw"])
    assert ref != 0.0
    assert abs(got - ref) <= 1e-12 * abs(ref), (got, ref)


def test_conv_exitbc_tasks(env):
    """Task 1 after each of u, v, w (and the p, sc1 calls, which change
    nothing), then task 2 for u, v, w: every field the calls write."""
    st = env
    s = state(st, 5)
    ref = s.to("numpy")
    g = s.to("torch")
    names = ("rho", "rhonp1", "u", "v", "w", "u_int", "v_int", "w_int", "hn_u", "hn_v", "hn_w")
    calls = [(1, iva) for iva in (1, 2, 3, 4, 5)] + [(2, iva) for iva in (1, 2, 3)]
    for task, iva in calls:
        st.orc.conv_exitbc(task, iva, 2e-3, *[ref[n] for n in names], st.m, st.dkp, st.dkw)
        L.conv_exitbc(task, iva, *[g[n] for n in names], g["metric"], g["dkp"], g["dkw"])
    got = g.to("numpy")
    for n in names[2:]:
        assert rel(got[n], ref[n]) <= 1e-12, (n, rel(got[n], ref[n]))
    # the outflow planes moved
    assert rel(ref["u_int"], s["u_int"]) > 1e-6


def test_fixed_inlet_bitwise(env):
    st = env
    s = state(st, 6)
    up, vp = profiles(st.case)
    ref = s.to("numpy")
    names = ("u_int", "v_int", "w_int", "u", "v", "w", "sc1", "rho")
    st.orc.fixed_inlet(INLET, up, vp, SEED, 7, 1.0, 1.0, ref["u"], ref["v"], ref["w"], ref["sc1"], ref["rho"],
                       ref["u_int"], ref["v_int"], ref["w_int"])
    L.gpu_set_inlet(INLET, up, vp, SEED)
    g = s.to("torch")
    L.fixed_inlet(*[g[n] for n in names], SEED, up, vp, 7)
    got = g.to("numpy")
    for n in names:
        np.testing.assert_array_equal(got[n], ref[n], err_msg=n)
    assert not np.array_equal(ref["u"], s["u"])


@pytest.mark.parametrize("exact", [1, 0])
def test_steps_inflow_outflow(exact, gpulib):
    """Three whole steps with the inflow and outflow sides, Smagorinsky,
    the reference solver."""
    st = setup()
    ctrl = L.default_ctrl(dtime=2e-3, model=1, exact=exact)
    s = S.new_state(st.case, st.m, st.dkp, st.dkw)
    S.init_channel(s, seed=8)
    up, vp = profiles(st.case)
    ref = s.to("numpy")
    st.orc.set_inlet(INLET, up, vp, SEED)
    mg, k = O.mgctrl_from_ctrl(ctrl), O.phys_from_ctrl(ctrl)
    for it in range(1, 4):
        st.orc.step(mg, k, it, it + 1, ref)
    L.gpu_init(st.case.geom(), ctrl)
    try:
        L.gpu_set_inlet(INLET, up, vp, SEED)
        g = s.to("torch")
        rcs = [S.step(g, it) for it in range(1, 4)]
        got = g.to("numpy")
    finally:
        L.gpu_finalize()
    assert rcs == [0, 0, 0]
    bad = {n: rel(got[n], ref[n]) for n in S.STATE if rel(got[n], ref[n]) > 1e-10}
    assert not bad, bad
    assert rel(got["u"], s["u"]) > 1e-6


@pytest.mark.parametrize("psolve", [L.PSOLVE_REFERENCE, L.PSOLVE_FP64])
def test_steps_six_blocks(psolve, gpulib):
    """The six-block boundary layer (two rows of uneven blocks joined by
    interfaces in x and y, two inlet blocks, two outlet blocks, a wall and
    a slip side), one eighth of its size: whole steps against the oracle,
    density ratio 1.5 carried by the scalar, Smagorinsky."""
    case = grid.bl6_case(8)
    cases.CASES["bl6"] = lambda: case
    try:
        st = cases.Setup("bl6", seed=3)
    finally:
        del cases.CASES["bl6"]
    ctrl = L.default_ctrl(dtime=2e-3, model=1, rholo=1.0, rhohi=1.5, psolve=psolve, rtol=1e-11, max_outer=100)
    s = S.new_state(case, st.m, st.dkp, st.dkw)
    S.init_bl6(s, rholo=1.0, rhohi=1.5)
    up, vp = grid.bl6_inflow(case)
    inlet = [1, 0, 0, 4]
    ref = s.to("numpy")
    st.orc.set_inlet(inlet, up, vp, SEED)
    mg = O.mgctrl_from_ctrl(ctrl) if psolve == L.PSOLVE_REFERENCE else O.mgctrl(nummgits=300, tolf=1e-15)
    k = O.phys_from_ctrl(ctrl)
    for it in range(1, 4):
        st.orc.step(mg, k, it, it + 1, ref)
    L.gpu_init(case.geom(), ctrl)
    try:
        L.gpu_set_inlet(inlet, up, vp, SEED)
        g = s.to("torch")
        rcs = [S.step(g, it) for it in range(1, 4)]
        got = g.to("numpy")
    finally:
        L.gpu_finalize()
    assert all(rc == 0 for rc in rcs), rcs
    tol = 1e-10 if psolve == L.PSOLVE_REFERENCE else 1e-7
    bad = {n: rel(got[n], ref[n]) for n in ("u", "v", "w", "sc1", "rho", "rhonp1") if rel(got[n], ref[n]) > tol}
    assert not bad, bad
    assert rel(got["u"], s["u"]) > 1e-6


def test_recycling_bitwise(gpulib):
    """The recycling-rescaling inflow on an eight-block chain: running
    means every step, rescaling at step 200, the plane copy; every array
    bitwise (the sums run in the reference's order on both sides)."""
    case = grid.chain_case(8, 6, 8, 4)
    cases.CASES["chain"] = lambda: case
    try:
        st = cases.Setup("chain", seed=3)
    finally:
        del cases.CASES["chain"]
    rng = np.random.default_rng(21)
    nprof = 32
    prof = [np.ascontiguousarray(1.0 + 0.1 * rng.random(nprof)) for _ in range(6)]
    means0 = [np.ascontiguousarray(0.5 + 0.1 * rng.random(nprof)) for _ in range(6)]
    s = state(st, 12)
    inlet = [0, 0, 1, 0]
    names = ("u", "v", "w", "sc1", "rho", "u_int", "v_int", "w_int")
    ref = s.to("numpy")
    rmeans = [m.copy() for m in means0]
    L.gpu_init(case.geom(), L.default_ctrl(rholo=1.0, rhohi=1.5))
    try:
        L.gpu_set_inlet(inlet, prof[0], prof[1], 0)
        g = s.to("torch")
        import torch
        gmeans = [torch.from_numpy(m.copy()).cuda() for m in means0]
        gprof = [torch.from_numpy(p).cuda() for p in prof]
        for step in (199, 200):
            st.orc.recycling(step, 1, inlet, 1.5, *[ref[n] for n in names], prof, rmeans)
            L.recycling(g["u_int"], g["v_int"], g["w_int"], g["u"], g["v"], g["w"], g["sc1"], g["rho"], gprof,
                        gmeans, step, 1)
        got = g.to("numpy")
        gm = [m.cpu().numpy() for m in gmeans]
    finally:
        L.gpu_finalize()
    for n in names:
        np.testing.assert_array_equal(got[n], ref[n], err_msg=n)
    for a, b in zip(gm, rmeans):
        np.testing.assert_array_equal(a, b)
    assert not np.array_equal(ref["u"], s["u"])


def test_statistics_bitwise(gpulib):
    """Span-averaged running statistics over two samples on the two-block
    inflow/outflow case: every 2-D output bitwise (same summation order)."""
    import torch
    st = setup()
    c = st.case
    s = state(st, 13)
    rng = np.random.default_rng(5)
    extra = {n: rng.standard_normal(c.n3_sg) for n in ("sc1var", "gam")}
    p = rng.standard_normal(c.n3_mg)
    outs0 = {n: 0.1 * rng.standard_normal(c.n2) for n in L.STAT_NAMES}
    ref = {n: a.copy() for n, a in outs0.items()}
    L.gpu_init(c.geom(), L.default_ctrl())
    try:
        dev = {n: torch.from_numpy(a.copy()).cuda() for n, a in outs0.items()}
        for no_sam in (1, 2):
            args = [s["u"], s["v"], s["w"], p, s["rho"], s["sc1"], extra["sc1var"], extra["gam"]]
            st.orc.statistics(no_sam, *args, ref)
            L.statistics(*[torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in args], dev, no_sam)
            s["u"] = s["u"] * 1.1
        got = {n: a.cpu().numpy() for n, a in dev.items()}
    finally:
        L.gpu_finalize()
    for n in L.STAT_NAMES:
        np.testing.assert_array_equal(got[n], ref[n], err_msg=n)
    assert not np.array_equal(ref["um"], outs0["um"])


@pytest.mark.parametrize("psolve,phys32", [(L.PSOLVE_FP64, 0), (L.PSOLVE_MIXED, 1)])
def test_six_blocks_step_graph(psolve, phys32, gpulib):
    """The six-block boundary layer with its inflow and outflow sides,
    steps 2..5 replayed from the whole-step graph (the inlet perturbation's
    step number read from device memory in the replay): the same fields as
    the steps launched call by call, bit for bit."""
    case = grid.bl6_case(8)
    cases.CASES["bl6"] = lambda: case
    try:
        st = cases.Setup("bl6", seed=3)
    finally:
        del cases.CASES["bl6"]
    up, vp = grid.bl6_inflow(case)
    inlet = [1, 0, 0, 4]
    s = S.new_state(case, st.m, st.dkp, st.dkw)
    S.init_bl6(s, rholo=1.0, rhohi=1.0)
    out = {}
    for graph in (0, 1):
        ctrl = L.default_ctrl(dtime=2e-3, model=1, psolve=psolve, rtol=1e-9, max_outer=100, exact=0,
                              phys32=phys32, step_graph=graph)
        L.gpu_init(case.geom(), ctrl)
        try:
            L.gpu_set_inlet(inlet, up, vp, SEED)
            g = s.to("torch")
            rcs = [S.step(g, it) for it in range(1, 6)]
            info = L.gpu_step_graph_info()
            L.gpu_sync()
            out[graph] = (g.to("numpy"), rcs, info)
        finally:
            L.gpu_finalize()
    (a, ra, _), (b, rb, info) = out[0], out[1]
    assert ra == rb == [0] * 5
    assert not info["failed"] and info["replays"] == 4, info
    for n in S.STATE:
        assert np.array_equal(a[n], b[n]), n
    assert rel(b["u"], s["u"]) > 1e-6
