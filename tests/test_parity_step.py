"""GPU parity of the momentum predictor (set_uv_int for u and v, set_w_int)
and of the scalar transport (set_gamsc1_bc, set_sc1, set_sc1_bc,
set_sc1var) against the oracle, through the C ABI.

Bar: relative 1e-13 where the reference calls log/pow (log-law wall
stress, filter width), bitwise everywhere else.  set_sc1 updates sc1 in
place in the reference's loop order; the GPU sweeps hyperplanes and must
reproduce it bitwise.
"""
import numpy as np
import pytest

from fortranutils_gb300 import grid
from fortranutils_gb300 import lester as L

import cases
import oracle_lib as O

pytestmark = pytest.mark.gpu

NAMES = list(cases.CASES)
K = dict(visc=1.0 / 2800.0, ylaminar=11.3, kappa=0.41, cwfun=5.2 * 0.41)


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    L.gpu_sync()
    return t.cpu().numpy()


@pytest.fixture(params=[(n, e) for e in (1, 0) for n in NAMES],
                ids=[f"{n}-{'exact' if e else 'fast'}" for e in (1, 0) for n in NAMES])
def env(request, gpulib):
    name, exact = request.param
    s = cases.Setup(name, seed=11)
    s.exact = exact
    L.gpu_init(s.case.geom(), L.default_ctrl(dtime=0.01, exact=exact, **K))
    L.gpu_set_iststep(5)
    yield s
    L.gpu_finalize()


def fields(s):
    r = s.rng
    n = s.case.n3_sg
    d = {k: r.standard_normal(n) for k in ("u", "v", "w", "p", "hu")}
    d["u"] += 1.0
    d["rho"] = r.uniform(0.8, 1.2, n)
    d["rhonp1"] = r.uniform(0.8, 1.2, n)
    d["gam"] = r.uniform(0.0, 1e-3, n)
    return d


def wall_arrays(s, kind):
    o = s.orc.sizes()
    n_ki, n_jk = o[7], o[8]
    n_ij = sum(a * b for (a, b, c) in s.case.levels[0])
    r = s.rng
    # both sides of the y+ = 11.3 switch occur
    if kind == "u":
        return [r.uniform(1e-6, 1e-2, n_ki), r.uniform(1e-6, 1e-2, n_ki),
                r.uniform(1e-6, 1e-2, n_ij), r.uniform(1e-6, 1e-2, n_ij)]
    if kind == "v":
        return [r.uniform(1e-6, 1e-2, n_jk), r.uniform(1e-6, 1e-2, n_jk),
                r.uniform(1e-6, 1e-2, n_ij), r.uniform(1e-6, 1e-2, n_ij)]
    return [r.uniform(1e-6, 1e-2, n_ki), r.uniform(1e-6, 1e-2, n_ki),
            r.uniform(1e-6, 1e-2, n_jk), r.uniform(1e-6, 1e-2, n_jk)]


def close(a, b, exact=1):
    """exact build: 1e-13 per element (log/pow may differ in the last bit);
    fast build: relative L2 1e-12 and 1e-9 per element above a floor."""
    if exact:
        np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-300)
        return
    scale = np.abs(b).max()
    assert np.linalg.norm(a - b) <= 1e-12 * max(np.linalg.norm(b), 1e-300)
    np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12 * scale)


@pytest.mark.parametrize("iva", [1, 2])
def test_set_uv_int(env, iva):
    s = env
    f = fields(s)
    tw = wall_arrays(s, "u" if iva == 1 else "v")
    a, b = (f["u"], f["v"]) if iva == 1 else (f["v"], f["u"])
    ui_ref, hu_ref = np.zeros(s.case.n3_sg), f["hu"].copy()
    tw_ref = [t.copy() for t in tw]
    s.orc.set_uv_int(iva, 0.01, 5, K, a, b, f["w"], f["p"], f["rho"], f["rhonp1"], f["gam"],
                     ui_ref, hu_ref, s.m, s.dkp, s.dkw, tw_ref)
    ui, hu = dev(np.zeros(s.case.n3_sg)), dev(f["hu"])
    twd = [dev(t) for t in tw]
    md = {k: dev(v) for k, v in s.m.items()}
    L.set_uv_int(iva, dev(a), dev(b), dev(f["w"]), dev(f["p"]), dev(f["rho"]), dev(f["rhonp1"]),
                 dev(f["gam"]), ui, hu, md, dev(s.dkp), dev(s.dkw), *twd)
    close(host(ui), ui_ref, s.exact)
    close(host(hu), hu_ref, s.exact)
    for q in range(4):
        close(host(twd[q]), tw_ref[q], s.exact)


def test_set_w_int(env):
    s = env
    f = fields(s)
    tw = wall_arrays(s, "w")
    wi_ref, hw_ref = np.zeros(s.case.n3_sg), f["hu"].copy()
    tw_ref = [t.copy() for t in tw]
    s.orc.set_w_int(0.01, 5, K, f["u"], f["v"], f["w"], f["p"], f["rho"], f["rhonp1"], f["gam"],
                    wi_ref, hw_ref, s.m, s.dkp, s.dkw, tw_ref)
    wi, hw = dev(np.zeros(s.case.n3_sg)), dev(f["hu"])
    twd = [dev(t) for t in tw]
    md = {k: dev(v) for k, v in s.m.items()}
    L.set_w_int(dev(f["u"]), dev(f["v"]), dev(f["w"]), dev(f["p"]), dev(f["rho"]),
                dev(f["rhonp1"]), dev(f["gam"]), wi, hw, md, dev(s.dkp), dev(s.dkw), *twd)
    close(host(wi), wi_ref, s.exact)
    close(host(hw), hw_ref, s.exact)
    for q in range(4):
        close(host(twd[q]), tw_ref[q], s.exact)


def test_scalar_transport(env):
    """set_gamsc1_bc -> set_sc1 (in-place, hyperplane order) -> set_sc1_bc;
    bitwise in the exact build."""
    s = env
    c = s.case
    r = s.rng
    n = c.n3_sg
    sc1 = r.uniform(0.0, 1.0, n)
    gs1 = r.uniform(0.0, 1e-3, n)
    gl = np.zeros(n)
    hs = r.standard_normal(n) * 1e-3
    u, v, w = (r.standard_normal(n) * 0.5 for _ in range(3))
    # exact zeros make the limiter take its third branch too
    u[::7] = 0.0
    rho = r.uniform(0.8, 1.2, n)
    g_ref, l_ref = gs1.copy(), gl.copy()
    s.orc.set_gamsc1_bc(K["visc"], sc1, g_ref, l_ref, s.m, s.dkp)
    sc_ref, hs_ref = sc1.copy(), hs.copy()
    s.orc.set_sc1(0.01, s.m, s.dkp, s.dkw, u, v, w, sc_ref, hs_ref, rho, g_ref, l_ref)
    s.orc.set_sc1_bc(sc_ref)
    md = {k: dev(val) for k, val in s.m.items()}
    gd, ld = dev(gs1), dev(gl)
    L.set_gamsc1_bc(dev(sc1), gd, ld, md["diu"], md["djv"], dev(s.dkp), md["rp"])
    assert np.array_equal(host(gd), g_ref) and np.array_equal(host(ld), l_ref)
    scd, hsd = dev(sc1), dev(hs)
    L.set_sc1(dev(u), dev(v), dev(w), None, scd, dev(rho), gd, ld, hsd, md, dev(s.dkp),
              dev(s.dkw))
    L.set_sc1_bc(scd)
    if s.exact:
        assert np.array_equal(host(scd), sc_ref)
        assert np.array_equal(host(hsd), hs_ref)
    else:
        close(host(scd), sc_ref, 0)
        close(host(hsd), hs_ref, 0)


def test_set_sc1var(env):
    s = env
    c = s.case
    sc1 = s.rng.uniform(0.0, 1.0, c.n3_sg)
    ref = np.zeros(c.n3_sg)
    s.orc.set_sc1var(sc1, ref, s.m, s.dkp, s.dkw)
    d = dev(np.zeros(c.n3_sg))
    md = {k: dev(val) for k, val in s.m.items()}
    L.set_sc1var(None, None, None, dev(sc1), None, d, None, md["dip"], md["djp"], dev(s.dkp),
                 dev(s.dkw), md["rp"])
    close(host(d), ref, s.exact)


def scalar_fields(case, rng):
    n = case.n3_sg
    sc1 = rng.uniform(0.0, 1.0, n)
    gs1 = rng.uniform(0.0, 1e-3, n)
    gl = np.full(n, 1e-4)
    hs = rng.standard_normal(n) * 1e-3
    u, v, w = (rng.standard_normal(n) * 0.5 for _ in range(3))
    u[::7] = 0.0
    rho = rng.uniform(0.8, 1.2, n)
    return sc1, gs1, gl, hs, u, v, w, rho


def run_sweep(case, m, dkp, dkw, f, ctrl):
    """set_gamsc1_bc then set_sc1 with the given controls; (sc1, hsc1)."""
    sc1, gs1, gl, hs, u, v, w, rho = f
    L.gpu_init(case.geom(), ctrl)
    try:
        md = {k: dev(val) for k, val in m.items()}
        gd, ld = dev(gs1), dev(gl)
        L.set_gamsc1_bc(dev(sc1), gd, ld, md["diu"], md["djv"], dev(dkp), md["rp"])
        scd, hsd = dev(sc1), dev(hs)
        L.set_sc1(dev(u), dev(v), dev(w), None, scd, dev(rho), gd, ld, hsd, md, dev(dkp), dev(dkw))
        return host(scd), host(hsd)
    finally:
        L.gpu_finalize()


SWEEP_CASES = {
    # the benchmarked layout at 1/16 of the cells: 30 layers of tiles
    "mixing64": lambda: grid.box_case(64, 48, 32, lx=7.5, ly=7.5, lz=3.75, ybc=L.BCT_ZERO_GRAD, beta=2.0),
    # more rows than one tile holds: two tiles per layer, chained in j
    "rows300": lambda: grid.box_case(12, 300, 6, ybc=L.BCT_WALL),
    # uneven blocks joined by interfaces (interface gradients at tile edges)
    "two_block": lambda: grid.two_block_case(12, 8, 8, 6),
}


@pytest.mark.parametrize("build", ["exact", "fast", "f32"])
@pytest.mark.parametrize("name", list(SWEEP_CASES))
def test_scalar_sweep_variants(name, build, gpulib):
    """The tile pipeline (ctrl.sc1_sweep 2), the hyperplane sweep (1) and
    per-plane launches (3) give the same in-place update: bitwise in the
    exact build and equal to the oracle; the fast and FP32 builds within
    rounding of the other two variants of the same build."""
    case = SWEEP_CASES[name]()
    orc = O.Oracle(case)
    x, y, z = case.coordinates()
    met, dkp, dkw = orc.comp_metric(x, y, z)
    m = cases.metrics_dict(met)
    f = scalar_fields(case, np.random.default_rng(17))
    kw = dict(dtime=0.01, **K)
    kw.update(exact=1) if build == "exact" else kw.update(exact=0, phys32=int(build == "f32"))
    got = {sw: run_sweep(case, m, dkp, dkw, f, L.default_ctrl(sc1_sweep=sw, **kw)) for sw in (1, 2, 3)}
    if build == "exact":
        for q in (0, 1):
            assert np.array_equal(got[1][q], got[3][q])
        sc1, gs1, gl, hs, u, v, w, rho = f
        g_ref, l_ref = gs1.copy(), gl.copy()
        orc.set_gamsc1_bc(K["visc"], sc1, g_ref, l_ref, m, dkp)
        sc_ref, hs_ref = sc1.copy(), hs.copy()
        orc.set_sc1(0.01, m, dkp, dkw, u, v, w, sc_ref, hs_ref, rho, g_ref, l_ref)
        assert np.array_equal(got[1][0], sc_ref) and np.array_equal(got[1][1], hs_ref)
        assert np.array_equal(got[2][0], sc_ref) and np.array_equal(got[2][1], hs_ref)
        return
    # the builds with FMA contraction: each variant's expression trees
    # contract differently, so they agree to rounding, not bitwise
    tol = 1e-12 if build == "fast" else 2e-6
    for other in (1, 3):
        for q in (0, 1):
            a, b = got[2][q], got[other][q]
            err = np.linalg.norm(a - b) / np.linalg.norm(b)
            assert err <= tol, (other, q, err)
