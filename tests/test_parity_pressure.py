"""GPU parity of the pressure path, halo exchange and metrics against the
oracle, through the C ABI.

Bar: bitwise for every routine whose arithmetic is the reference's operation
for operation (metrics, coeff_p, sour_p, residual, transfers, lexicographic
SOR, lmg_solve in reference mode, extrap_p, p_ref_subtract, uvw_adv,
swap_sc, density update, slip faces).  Norms are sums in a different order:
relative 1e-12.  The fast solvers (red-black FP64 and mixed FP32/FP64) are a
different algorithm: their solution must match a tightly converged
reference-mode solution to relative L2 <= 1e-6 after p_ref_subtract, and
their own residual must reach the requested 1e-9.
"""
import numpy as np
import pytest

from fortranutils_gb300 import lester as L

import cases
import oracle_lib as O

pytestmark = pytest.mark.gpu

NAMES = list(cases.CASES)


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    L.gpu_sync()
    return t.cpu().numpy()


@pytest.fixture(params=NAMES)
def env(request, gpulib):
    s = cases.Setup(request.param, seed=7)
    L.gpu_init(s.case.geom(), L.default_ctrl(dtime=0.01))
    yield s
    L.gpu_finalize()


def gpu_metrics(s):
    c = s.case
    m = {n: dev(np.zeros(c.n2)) for n in L.METRIC_NAMES}
    dkp, dkw = dev(np.zeros(c.n1k)), dev(np.zeros(c.n1k))
    L.comp_metric(dev(s.x), dev(s.y), dev(s.z), m, dkp, dkw)
    return {k: host(v) for k, v in m.items()}, host(dkp), host(dkw)


def test_sizes_match_oracle(env):
    s = env
    z = L.gpu_sizes()
    o = s.orc.sizes()
    assert (z.nummgl, z.n3_mg, z.n3_sg, z.n2, z.n1k, z.nxy, z.nz) == tuple(o[:7])
    for lev in range(1, z.nummgl + 1):
        for ib in range(1, len(s.case.blocks) + 1):
            n, off = L.gpu_block_info(lev, ib)
            on, _, oo = s.orc.block_info(lev, ib)
            assert n == on and off[:5] == oo[:5]


def test_comp_metric_bitwise(env):
    s = env
    m, dkp, dkw = gpu_metrics(s)
    for n in L.METRIC_NAMES:
        assert np.array_equal(m[n], s.m[n]), n
    assert np.array_equal(dkp, s.dkp) and np.array_equal(dkw, s.dkw)


def test_coeff_p_bitwise(env):
    s = env
    c = s.case
    a = [dev(np.zeros(c.n3_mg)) for _ in range(7)]
    md = {k: dev(v) for k, v in s.m.items()}
    L.coeff_p(md["diu"], md["djv"], md["rdiv"], md["rdju"], md["didjp"], md["rp"], dev(s.dkp),
              dev(s.dkw), *a)
    for q in range(7):
        assert np.array_equal(host(a[q]), s.a[q]), q


def test_coeff_p_host_arrays(env):
    """Strict drop-in mode: numpy (host) arrays in and out."""
    s = env
    c = s.case
    a = [np.zeros(c.n3_mg) for _ in range(7)]
    L.coeff_p(s.m["diu"], s.m["djv"], s.m["rdiv"], s.m["rdju"], s.m["didjp"], s.m["rp"], s.dkp,
              s.dkw, *a)
    for q in range(7):
        assert np.array_equal(a[q], s.a[q]), q


def test_swap_sc_bitwise(env):
    s = env
    f = s.interior_random(mg=True, ghosts=True)
    for lev in range(1, s.case.nummgl + 1):
        ref = f.copy()
        s.orc.swap_sc(lev, ref, 1)
        d = dev(f)
        L.swap_sc(L.SV_P, lev, d)
        assert np.array_equal(host(d), ref), lev


def test_norms_bitwise_residual(env):
    s = env
    x = s.interior_random(mg=True, ghosts=True)
    b = s.interior_random(mg=True)
    for lev in range(1, s.case.nummgl + 1):
        r_ref = np.zeros(s.case.n3_mg)
        n_ref = s.orc.norms(lev, 1, s.a, x, b, r_ref)
        rd = dev(np.zeros(s.case.n3_mg))
        n_gpu = L.norms(lev, 1, *[dev(a) for a in s.a], dev(x), dev(b), rd)
        assert np.array_equal(host(rd), r_ref)
        np.testing.assert_allclose(n_gpu, n_ref, rtol=1e-12)


def test_restriction_prolongation_bitwise(env):
    s = env
    c = s.case
    if c.nummgl < 2:
        pytest.skip("single level")
    f = s.interior_random(mg=True, ghosts=True)
    for lev in range(2, c.nummgl + 1):
        f1 = s.interior_random(mg=True)
        ref = f1.copy()
        s.orc.restriction(lev, f, ref)
        d = dev(f1)
        L.restriction(lev, dev(f), d)
        assert np.array_equal(host(d), ref), lev
    for lev in range(1, c.nummgl):
        ref = f.copy()
        s.orc.prolongation(lev, ref)
        d = dev(f)
        L.prolongation(lev, d)
        assert np.array_equal(host(d), ref), lev


@pytest.mark.parametrize("jumble", [0, 8, 13, 21, 95])
def test_sporlx_bitwise(env, jumble):
    """Every pass direction (jumble rotation) and level."""
    s = env
    b = s.interior_random(mg=True)
    for lev in range(1, s.case.nummgl + 1):
        f = s.interior_random(mg=True)
        s.orc.set_jumble(jumble)
        ref = f.copy()
        n_ref = s.orc.sporlx(lev, s.a, ref, b, 1.6, 0.0, (0.0, 1.0, 1.0, 1.0))
        L.gpu_set_jumble(jumble)
        d = dev(f)
        n_gpu = L.sporlx(lev, *[dev(a) for a in s.a], d, dev(b), 1.6, 0.0, (0.0, 1.0, 1.0, 1.0))
        assert np.array_equal(host(d), ref), (lev, jumble)
        assert L.gpu_get_jumble() == s.orc.get_jumble()
        np.testing.assert_allclose(np.array(n_gpu)[[0, 2, 3]], np.array(n_ref)[[0, 2, 3]],
                                   rtol=1e-12)


@pytest.mark.parametrize("cycle", [1, 2])
def test_lmg_solve_reference_bitwise(env, cycle):
    """lmg_solve in reference mode: same V/F-cycle schedule, same SOR order."""
    s = env
    c = s.case
    b = s.interior_random(mg=True, zero_mean=True)
    f = np.zeros(c.n3_mg)
    ctrl = L.default_ctrl(psolve=L.PSOLVE_REFERENCE, nummgits=5, meth_cycle=cycle)
    L.gpu_set_ctrl(ctrl)
    fr, br, rr = f.copy(), b.copy(), np.zeros(c.n3_mg)
    s.orc.set_jumble(0)
    out = s.orc.lmg_solve(O.mgctrl(nummgits=5, meth_cycle=cycle), s.a, fr, br, rr)
    L.gpu_set_jumble(0)
    fd, bd, rd = dev(f), dev(b), dev(np.zeros(c.n3_mg))
    L.lmg_solve(*[dev(a) for a in s.a], fd, bd, rd)
    st = L.gpu_solve_stats()
    assert np.array_equal(host(fd), fr)
    assert np.array_equal(host(bd), br)
    assert np.array_equal(host(rd), rr)
    assert st["cycles"] == int(out[4])
    np.testing.assert_allclose([st["rnorm"], st["fnorm"], st["enorm"], st["vnorm"]], out[:4],
                               rtol=1e-12)


@pytest.mark.parametrize("layout", ["tail", "per-level", "stored-coef"])
@pytest.mark.parametrize("psolve", [L.PSOLVE_FP64, L.PSOLVE_MIXED])
def test_fast_solvers_converge_to_reference(env, psolve, layout):
    """The fast solvers reach the converged reference solution, with the
    coarse levels in one single-CTA launch (default on these small grids),
    with one launch per operation, and with stored FP32 coefficients."""
    s = env
    c = s.case
    b = s.interior_random(mg=True, zero_mean=True)
    # reference-mode solution converged to the FP64 floor
    fr, br, rr = np.zeros(c.n3_mg), b.copy(), np.zeros(c.n3_mg)
    s.orc.set_jumble(0)
    s.orc.lmg_solve(O.mgctrl(nummgits=400, tolf=1e-15), s.a, fr, br, rr)
    s.orc.p_ref_subtract(fr)
    ctrl = L.default_ctrl(psolve=psolve, rtol=1e-9, max_outer=400,
                          mg_tail=0 if layout != "tail" else 32768,
                          rb_matfree=0 if layout == "stored-coef" else 1)
    L.gpu_set_ctrl(ctrl)
    fd, bd, rd = dev(np.zeros(c.n3_mg)), dev(b), dev(np.zeros(c.n3_mg))
    L.lmg_solve(*[dev(a) for a in s.a], fd, bd, rd)
    st = L.gpu_solve_stats()
    assert st["relres"] <= 1e-9
    L.p_ref_subtract(fd)
    got = host(fd)[: c.n3_sg]
    ref = fr[: c.n3_sg]
    inner = np.zeros(c.n3_sg, dtype=bool)
    for ib in range(len(c.blocks)):
        c.block_view(inner, ib)[1:-1, 1:-1, 1:-1] = True
    err = np.linalg.norm(got[inner] - ref[inner]) / np.linalg.norm(ref[inner])
    assert err <= 1e-6, err


def test_extrap_p_and_p_ref_bitwise(env):
    s = env
    p = s.interior_random(ghosts=True)
    ref = p.copy()
    s.orc.extrap_p(ref)
    s.orc.p_ref_subtract(ref)
    d = dev(p)
    L.extrap_p(d)
    L.p_ref_subtract(d)
    assert np.array_equal(host(d), ref)


def test_sour_p_bitwise(env):
    s = env
    c = s.case
    u, v, w = (s.interior_random(ghosts=True) for _ in range(3))
    rho, rhonp1 = s.positive(), s.positive()
    outs = [np.zeros(c.n3_sg) for _ in range(4)]
    s.orc.sour_p(0.01, s.m, s.dkp, s.dkw, u, v, w, rho, rhonp1, outs)
    od = [dev(np.zeros(c.n3_sg)) for _ in range(4)]
    md = {k: dev(val) for k, val in s.m.items()}
    L.sour_p(md["diu"], md["djv"], md["rdiv"], md["rdju"], md["didjp"], dev(s.dkp), md["rdidjp"],
             dev(s.dkw), dev(u), dev(v), dev(w), dev(rho), dev(rhonp1), *od)
    for q in range(4):
        assert np.array_equal(host(od[q]), outs[q]), q


@pytest.mark.parametrize("ivar", [1, 2, 3])
def test_uvw_adv_bitwise(env, ivar):
    s = env
    u = s.interior_random(ghosts=True)
    ui = s.interior_random(ghosts=True)
    p = s.interior_random(ghosts=True)
    rho = s.positive()
    dg = s.m["djv"] if ivar == 2 else s.m["diu"]
    ref = u.copy()
    s.orc.uvw_adv(ivar, 0.01, dg, s.m["rp"], s.dkw, ref, ui, rho, p)
    d = dev(u)
    L.uvw_adv(ivar, dev(dg), dev(s.m["rp"]), dev(s.dkw), d, dev(ui), dev(rho), dev(p))
    assert np.array_equal(host(d), ref)


def test_density_update_bitwise(env):
    s = env
    sc1 = s.rng.uniform(-0.1, 1.1, s.case.n3_sg)
    rho = s.positive()
    rhonp1 = np.zeros(s.case.n3_sg)
    r_s, r_r = sc1.copy(), rhonp1.copy()
    s.orc.search_lib(r_s, r_r, 0.3, rho, 1.0, 2.0)
    ds, dr = dev(sc1), dev(rhonp1)
    L.search_lib(ds, None, dr, None, 1, 0.3, dev(rho), 1.0, 2.0)
    assert np.array_equal(host(ds), r_s) and np.array_equal(host(dr), r_r)
    rm1 = np.zeros(s.case.n3_sg)
    a, b_, c_ = rho.copy(), r_r.copy(), rm1.copy()
    s.orc.swap_rhos(a, b_, c_)
    da, db, dc = dev(rho), dev(r_r), dev(rm1)
    L.swap_rhos(da, db, dc)
    assert np.array_equal(host(da), a) and np.array_equal(host(dc), c_)


def test_slipbc_bitwise(env):
    s = env
    f = [s.interior_random(ghosts=True) for _ in range(5)]
    p = s.interior_random(ghosts=True)
    vint = s.interior_random(ghosts=True)
    ref = [a.copy() for a in f]
    s.orc.slipbc(0.01, s.m["djp"], ref[0], ref[1], vint, ref[2], ref[3], ref[4], p)
    d = [dev(a) for a in f]
    L.slipbc(None, None, None, None, None, dev(s.m["djp"]), None, None, d[0], d[1], dev(vint), d[2],
             d[3], d[4], dev(p))
    for q in range(5):
        assert np.array_equal(host(d[q]), ref[q]), q


@pytest.mark.parametrize("exact", [1, 0])
@pytest.mark.parametrize("model", [0, 1, 2, 3])
def test_subgrid(env, model, exact):
    """exact build: 1e-13 per element (pow may differ in the last bit);
    fast build (reciprocal tables, sqrt-based WALE powers, split filter
    width): relative L2 1e-12."""
    s = env
    c = s.case
    u, v, w = (s.interior_random(ghosts=True) for _ in range(3))
    sc1 = s.rng.uniform(0, 1, c.n3_sg)
    vdd = s.rng.uniform(0.5, 1.0, c.n3_sg)
    outs = [np.zeros(c.n3_sg) for _ in range(4)]
    # Sigma (model 3) takes the square root of the density relaxation
    # factor alpha; 0.3 gives non-zero viscosities
    alpha = 0.3 if model == 3 else 0.0
    s.orc.subgrid(model, 0.1, 0, outs[0], outs[1], u, v, w, sc1, outs[2], outs[3], vdd, s.m,
                  s.dkp, s.dkw, alpha)
    L.gpu_set_ctrl(L.default_ctrl(model=model, csles=0.1, exact=exact, alpha=alpha))
    od = [dev(np.zeros(c.n3_sg)) for _ in range(4)]
    md = {k: dev(val) for k, val in s.m.items()}
    L.subgrid(od[0], od[1], dev(u), dev(v), dev(w), dev(sc1), None, od[2], od[3], dev(vdd),
              md["dip"], md["diu"], md["djp"], md["djv"], dev(s.dkp), dev(s.dkw), md["hijp"],
              md["hjip"], md["hkip"], md["hkjp"], md["rp"])
    for q in range(4):
        got = host(od[q])
        if exact and model != 3:
            np.testing.assert_allclose(got, outs[q], rtol=1e-13, atol=1e-300)
        else:
            # Sigma: acos, cos and fractional powers (CUDA's against the
            # C library's) in a formula that cancels where two singular
            # values are close: relative L2 1e-10 over the finite values
            fin = np.isfinite(outs[q])
            assert np.array_equal(fin, np.isfinite(got)), q
            ref = outs[q][fin]
            tol = 1e-10 if model == 3 else 1e-12
            assert np.linalg.norm(got[fin] - ref) <= tol * max(np.linalg.norm(ref), 1e-300), q
    if model == 3:
        assert np.nanmax(np.abs(outs[0])) > 0


@pytest.mark.parametrize("psolve", [L.PSOLVE_FP64, L.PSOLVE_MIXED])
@pytest.mark.parametrize("krylov,line", [(1, 0), (2, 0), (2, 1)])
def test_fast_solvers_stretched_channel(psolve, krylov, line, gpulib):
    """A wall-stretched channel (tanh beta 2.2, 64x48x32): with a random
    right-hand side the plain defect-correction cycle converges slowly or
    not at all here (the coarse-grid correction overshoots near the
    walls); flexible CG, and the automatic switch to it, reach 1e-10 and
    the converged reference solution."""
    from fortranutils_gb300 import grid
    case = grid.box_case(64, 48, 32, ybc=L.BCT_WALL, beta=2.2)
    cases.CASES["stretched_channel"] = lambda: case
    try:
        s = cases.Setup("stretched_channel", seed=3)
    finally:
        del cases.CASES["stretched_channel"]
    b = s.interior_random(mg=True, zero_mean=True)
    fr, rr = np.zeros(case.n3_mg), np.zeros(case.n3_mg)
    s.orc.set_jumble(0)
    s.orc.lmg_solve(O.mgctrl(nummgits=120, tolf=1e-15), s.a, fr, b.copy(), rr)
    s.orc.p_ref_subtract(fr)
    ctrl = L.default_ctrl(psolve=psolve, rtol=1e-10, max_outer=60, krylov=krylov, rb_line=line)
    if line:
        ctrl.rb_omega, ctrl.rb_sweeps = 1.0, 2
    L.gpu_init(case.geom(), ctrl)
    try:
        fd = dev(np.zeros(case.n3_mg))
        L.lmg_solve(*[dev(a) for a in s.a], fd, dev(b), dev(np.zeros(case.n3_mg)))
        st = L.gpu_solve_stats()
        assert st["relres"] <= 1e-10 and st["cycles"] <= 40, st
        L.p_ref_subtract(fd)
        got = host(fd)[: case.n3_sg]
    finally:
        L.gpu_finalize()
    inner = np.zeros(case.n3_sg, dtype=bool)
    case.block_view(inner, 0)[1:-1, 1:-1, 1:-1] = True
    ref = fr[: case.n3_sg]
    err = np.linalg.norm(got[inner] - ref[inner]) / np.linalg.norm(ref[inner])
    assert err <= 1e-7, err


@pytest.mark.parametrize("psolve", [L.PSOLVE_FP64, L.PSOLVE_MIXED])
def test_fast_solvers_independent_boxes(psolve, gpulib):
    """Three unlinked boxes of uneven sizes in one solve (one launch per
    operation covers all of them): each box's operator is singular on its
    own, so each gets its own mean removed; every box matches its converged
    reference solution up to its own constant."""
    from fortranutils_gb300 import grid
    case = grid.boxes_case([(16, 8, 8), (8, 16, 8), (24, 8, 16)])
    cases.CASES["boxes3"] = lambda: case
    try:
        s = cases.Setup("boxes3", seed=4)
    finally:
        del cases.CASES["boxes3"]
    b = np.zeros(case.n3_mg)
    rng = np.random.default_rng(11)
    for ib in range(len(case.blocks)):
        v = case.block_view(b, ib, 0)[1:-1, 1:-1, 1:-1]
        v[...] = rng.standard_normal(v.shape)
        v -= v.mean()
    fr, rr = np.zeros(case.n3_mg), np.zeros(case.n3_mg)
    s.orc.set_jumble(0)
    s.orc.lmg_solve(O.mgctrl(nummgits=300, tolf=1e-15), s.a, fr, b.copy(), rr)
    L.gpu_init(case.geom(), L.default_ctrl(psolve=psolve, rtol=1e-10, max_outer=100))
    try:
        fd = dev(np.zeros(case.n3_mg))
        L.lmg_solve(*[dev(a) for a in s.a], fd, dev(b), dev(np.zeros(case.n3_mg)))
        st = L.gpu_solve_stats()
        assert st["relres"] <= 1e-10, st
        got = host(fd)
    finally:
        L.gpu_finalize()
    for ib in range(len(case.blocks)):
        g = case.block_view(got, ib, 0)[1:-1, 1:-1, 1:-1]
        r = case.block_view(fr, ib, 0)[1:-1, 1:-1, 1:-1]
        g, r = g - g.mean(), r - r.mean()
        assert np.linalg.norm(g - r) <= 1e-7 * np.linalg.norm(r), ib


@pytest.mark.parametrize("psolve", [L.PSOLVE_FP64, L.PSOLVE_MIXED])
def test_autotune(psolve, gpulib):
    """The first solve with autotune tries the candidate settings on the
    system itself, keeps the fastest converged one and still returns the
    converged solution; later solves use the chosen settings."""
    s = cases.Setup("box_wall", seed=5)
    c = s.case
    b = s.interior_random(mg=True, zero_mean=True)
    L.gpu_init(c.geom(), L.default_ctrl(psolve=psolve, rtol=1e-10, max_outer=200, autotune=1))
    try:
        prec = 64 if psolve == L.PSOLVE_FP64 else 32
        assert not L.gpu_tuned(prec)["done"]
        sols = []
        for _ in range(2):
            fd = dev(np.zeros(c.n3_mg))
            L.lmg_solve(*[dev(a) for a in s.a], fd, dev(b), dev(np.zeros(c.n3_mg)))
            assert L.gpu_solve_stats()["relres"] <= 1e-10
            L.p_ref_subtract(fd)
            sols.append(host(fd))
        t = L.gpu_tuned(prec)
    finally:
        L.gpu_finalize()
    assert t["done"]
    assert t["rb_threads"] in (128, 256, 512) and t["rb_sweeps"] in (1, 2, 3, 4)
    assert t["rb_omega"] in (1.0, 1.2, 1.3, 1.5) and t["mg_tail"] in (0, 1024, 4096, 16384)
    assert t["rb_line"] in (0, 1)
    assert np.linalg.norm(sols[0] - sols[1]) <= 1e-8 * np.linalg.norm(sols[1])
