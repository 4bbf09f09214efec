"""Failure detection through the C ABI, in forms that fault, trap or hang no
GPU: a bounded device wait made to run out (ctrl.wait_limit), NaN injected
into a host-built field, and a pressure system with a zero diagonal built on
the host.  Every case must return its LES_ERR_* code, and the library must
stay usable: the same call with good inputs afterwards gives the oracle's
result.

The reference stops on bad configuration (code/solvers.F:35-36,
code/smooth.F:77-79); a NaN or a zero diagonal there propagates through the
SOR updates (code/sporlx.F:243-272) into the norms of code/norms.F:118-121.
"""
import numpy as np
import pytest

from fortranutils_gb300 import lester as L
from fortranutils_gb300 import state as S

import cases
import oracle_lib as O

pytestmark = pytest.mark.gpu

ERR_NONFINITE, ERR_TIMEOUT = -6, -9


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    L.gpu_sync()
    return t.cpu().numpy()


def scalar_inputs(s):
    r = s.rng
    n = s.case.n3_sg
    sc1 = r.uniform(0.0, 1.0, n)
    gs1 = r.uniform(0.0, 1e-3, n)
    gl = np.zeros(n)
    hs = r.standard_normal(n) * 1e-3
    u, v, w = (r.standard_normal(n) * 0.5 for _ in range(3))
    rho = r.uniform(0.8, 1.2, n)
    return sc1, gs1, gl, hs, u, v, w, rho


@pytest.mark.parametrize("sweep", [1, 2])
def test_sweep_wait_times_out_then_recovers(sweep, gpulib):
    """A wait limit of one poll makes the scalar sweep's bounded wait (grid
    barrier, or a tile's wait on the tile before it) give up: LES_ERR_TIMEOUT.
    The same call with the default limit then matches the oracle bitwise."""
    s = cases.Setup("box_slip_stretched", seed=31)
    sc1, gs1, gl, hs, u, v, w, rho = scalar_inputs(s)
    K = dict(dtime=0.01, exact=1, sc1_sweep=sweep)
    L.gpu_init(s.case.geom(), L.default_ctrl(wait_limit=1, **K))
    try:
        md = {k: dev(val) for k, val in s.m.items()}
        gd, ld = dev(gs1), dev(gl)
        L.set_gamsc1_bc(dev(sc1), gd, ld, md["diu"], md["djv"], dev(s.dkp), md["rp"])
        args = (dev(u), dev(v), dev(w), None)
        with pytest.raises(L.LesterError) as ei:
            L.set_sc1(*args, dev(sc1), dev(rho), gd, ld, dev(hs), md, dev(s.dkp), dev(s.dkw))
        assert ei.value.code == ERR_TIMEOUT, ei.value
        L.gpu_set_ctrl(L.default_ctrl(wait_limit=0, **K))
        scd, hsd = dev(sc1), dev(hs)
        L.set_sc1(*args, scd, dev(rho), gd, ld, hsd, md, dev(s.dkp), dev(s.dkw))
        got_s, got_h = host(scd), host(hsd)
    finally:
        L.gpu_finalize()
    g_ref, l_ref = gs1.copy(), gl.copy()
    s.orc.set_gamsc1_bc(1.0 / 2800.0, sc1, g_ref, l_ref, s.m, s.dkp)
    sc_ref, hs_ref = sc1.copy(), hs.copy()
    s.orc.set_sc1(0.01, s.m, s.dkp, s.dkw, u, v, w, sc_ref, hs_ref, rho, g_ref, l_ref)
    assert np.array_equal(got_s, sc_ref)
    assert np.array_equal(got_h, hs_ref)


def _channel(psolve, **kw):
    st = cases.Setup("box_wall")
    ctrl = L.default_ctrl(dtime=2e-3, model=1, psolve=psolve, rtol=1e-10, **kw)
    s = S.new_state(st.case, st.m, st.dkp, st.dkw)
    S.init_channel(s, seed=5)
    return st, ctrl, s


@pytest.mark.parametrize("psolve", [L.PSOLVE_REFERENCE, L.PSOLVE_FP64, L.PSOLVE_MIXED])
def test_nan_in_a_field_is_reported(psolve, gpulib):
    """NaN written by the host into one interior u value: the step's pressure
    solve sees a non-finite residual and lester_step returns
    LES_ERR_NONFINITE.  A step of the clean fields then runs."""
    kw = dict(exact=0, phys32=1) if psolve == L.PSOLVE_MIXED else {}
    st, ctrl, s = _channel(psolve, **kw)
    bad = s.to("numpy")
    c = st.case
    c.block_view(bad["u"], 0)[5, 4, 6] = np.nan
    L.gpu_init(c.geom(), ctrl)
    try:
        g = bad.to("torch")
        with pytest.raises(L.LesterError) as ei:
            S.step(g, 1)
        assert ei.value.code == ERR_NONFINITE, ei.value
        good = s.to("torch")
        assert S.step(good, 1) == 0
        got = good.to("numpy")
    finally:
        L.gpu_finalize()
    assert all(np.isfinite(got[n]).all() for n in ("u", "v", "w", "p"))


@pytest.mark.parametrize("psolve", [L.PSOLVE_REFERENCE, L.PSOLVE_FP64, L.PSOLVE_MIXED])
def test_zero_diagonal_is_reported(psolve, gpulib):
    """A pressure system whose ap is zero at one interior point (built on the
    host): the solve returns LES_ERR_NONFINITE.  The intact system then
    solves to its tolerance."""
    st = cases.Setup("box_wall", seed=41)
    c = st.case
    bsrc = st.interior_random(mg=True, zero_mean=True)
    a_bad = [x.copy() for x in st.a]
    c.block_view(a_bad[0], 0)[6, 3, 5] = 0.0
    L.gpu_init(c.geom(), L.default_ctrl(psolve=psolve, rtol=1e-10, nummgits=50, tolf=1e-14))
    try:
        p = dev(np.zeros(c.n3_mg))
        res = dev(np.zeros(c.n3_mg))
        with pytest.raises(L.LesterError) as ei:
            L.lmg_solve(*[dev(x) for x in a_bad], p, dev(bsrc), res)
        assert ei.value.code == ERR_NONFINITE, ei.value
        p = dev(np.zeros(c.n3_mg))
        L.lmg_solve(*[dev(x) for x in st.a], p, dev(bsrc), res)
        stats = L.gpu_solve_stats()
    finally:
        L.gpu_finalize()
    if psolve == L.PSOLVE_REFERENCE:
        assert np.isfinite(stats["rnorm"]) and stats["rnorm"] < 1e-6 * stats["fnorm"]
    else:
        assert stats["relres"] <= 1e-10
