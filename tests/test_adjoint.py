"""Adjoint and tangent-linear runs of the time step (lester_adjoint_run,
lester_tangent_run) on small channels, through the C ABI.

Objective: the mean wall shear stress over a window of steps; control: the
body force of the u, v, w predictors.  Runs without an eddy-viscosity model
and with the Smagorinsky model (model 1: gam, its van Driest damping in the
wall-stress running means and the wall ghosts are differentiated).  Checks:
  * the tangent against central finite differences of the forward run
    (relative 1e-6: the O(eps^2) truncation of a quadratic map);
  * the adjoint gradient against the tangent along random directions
    (<grad J, d> = dJ(d), relative 1e-9: the two runs differ only by the
    rounding and the 1e-12 residuals of their pressure solves);
  * the gradient does not depend on the checkpoint interval;
  * the caller's state is left unchanged, and runs outside the scope the
    transposition covers are refused.
"""
import numpy as np
import pytest

from fortranutils_gb300 import lester as L
from fortranutils_gb300 import state as S

import cases

pytestmark = pytest.mark.gpu

NSTEP = 4


def start(name, psolve=L.PSOLVE_FP64, **kw):
    """A channel state after one ordinary step (which forms the pressure
    coefficients and the wall-stress running means), laminar at the walls."""
    import torch
    st = cases.Setup(name)
    ctrl = dict(dtime=2e-3, model=0, psolve=psolve, rtol=1e-12, max_outer=400, visc=1.0 / 500.0)
    ctrl.update(kw)
    s = S.new_state(st.case, st.m, st.dkp, st.dkw)
    S.init_channel(s, seed=7)
    g = s.to("torch")
    L.gpu_init(st.case.geom(), L.default_ctrl(**ctrl))
    assert S.step(g, 1) == 0
    torch.cuda.synchronize()
    return st, g


def direction(st, seed):
    """A body-force direction: a uniform streamwise part plus noise."""
    import torch
    rng = np.random.default_rng(seed)
    st.rng = rng
    du = st.interior_random(scale=0.3)
    for ib in range(len(st.case.blocks)):
        st.case.block_view(du, ib, 0)[1:-1, 1:-1, 1:-1] += 1.0
    dv = st.interior_random(scale=0.3)
    dw = st.interior_random(scale=0.3)
    return [torch.from_numpy(a).cuda() for a in (du, dv, dw)]


def dot(a, b):
    return float(sum((x * y).sum().item() for x, y in zip(a, b)))


@pytest.fixture
def finalize():
    yield
    L.gpu_finalize()


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("name", ["box_wall", "two_block"])
def test_tangent_matches_finite_differences(name, model, finalize):
    import torch
    st, g = start(name, model=model)
    if model == 1:  # the eddy viscosity is comparable to the molecular one
        assert g["gam"].abs().max().item() > 0.5 / 500.0
    d = direction(st, 11)
    J0, dJ = S.tangent_run(g, NSTEP, *d, j_first=2)
    assert J0 > 0 and dJ != 0
    eps = 1e-3
    Js = []
    for sgn in (1.0, -1.0):
        f = [sgn * eps * x for x in d]
        L.gpu_set_body_force(*f)
        zero = [torch.zeros_like(x) for x in d]
        Js.append(S.tangent_run(g, NSTEP, *zero, j_first=2)[0])
        L.gpu_set_body_force()
    fd = (Js[0] - Js[1]) / (2 * eps)
    assert abs(fd - dJ) <= 1e-6 * abs(dJ), (fd, dJ)


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("psolve", [L.PSOLVE_FP64, L.PSOLVE_MIXED])
@pytest.mark.parametrize("name", ["box_wall", "two_block"])
def test_adjoint_matches_tangent(name, psolve, model, finalize):
    """The adjoint is the transpose of the tangent: for two directions,
    <grad J, d> equals the tangent's dJ(d)."""
    import torch
    st, g = start(name, psolve=psolve, model=model)
    grad = [torch.zeros_like(g["u"]) for _ in range(3)]
    J = S.adjoint_run(g, NSTEP, *grad, j_first=2, checkpoint=2)
    for seed in (3, 4):
        d = direction(st, seed)
        Jt, dJ = S.tangent_run(g, NSTEP, *d, j_first=2)
        assert abs(Jt - J) <= 1e-12 * abs(J)
        adj = dot(grad, d)
        assert abs(adj - dJ) <= 1e-9 * abs(dJ), (adj, dJ)


@pytest.mark.parametrize("model", [0, 1])
def test_gradient_independent_of_checkpoints(model, finalize):
    import torch
    st, g = start("box_wall", model=model)
    out = []
    for K in (1, 3, NSTEP):
        grad = [torch.zeros_like(g["u"]) for _ in range(3)]
        J = S.adjoint_run(g, NSTEP, *grad, checkpoint=K)
        out.append((J, [x.cpu().numpy() for x in grad]))
    J0, g0 = out[0]
    scale = max(np.abs(x).max() for x in g0)
    assert scale > 0
    for J, gk in out[1:]:
        assert abs(J - J0) <= 1e-14 * abs(J0)
        for a, b in zip(gk, g0):
            assert np.abs(a - b).max() <= 1e-12 * scale


def test_window_and_state_unchanged(finalize):
    """A window of one step; the caller's arrays are not touched."""
    import torch
    st, g = start("box_wall")
    before = {n: g[n].clone() for n in S.STATE}
    grad = [torch.zeros_like(g["u"]) for _ in range(3)]
    J_last = S.adjoint_run(g, NSTEP, *grad, j_first=NSTEP, j_last=NSTEP)
    d = direction(st, 5)
    Jt, dJ = S.tangent_run(g, NSTEP, *d, j_first=NSTEP, j_last=NSTEP)
    assert abs(Jt - J_last) <= 1e-12 * abs(J_last)
    assert abs(dot(grad, d) - dJ) <= 1e-9 * abs(dJ)
    for n in S.STATE:
        assert torch.equal(g[n], before[n]), n
    # the gradient vanishes where the predictors write nothing: the first
    # interior v plane on each wall
    gv = grad[1].cpu().numpy()
    for ib in range(len(st.case.blocks)):
        assert np.all(st.case.block_view(gv, ib, 0)[:, 1, :] == 0.0)


@pytest.mark.parametrize("name,bad", [("box_wall", dict(model=2)), ("box_wall", dict(model=3)),
                                      ("box_wall", dict(rholo=1.0, rhohi=2.0)),
                                      ("box_wall", dict(psolve=L.PSOLVE_REFERENCE)),
                                      ("box_slip_stretched", {})])
def test_scope_refused(name, bad, finalize):
    """WALE and Sigma eddy viscosity, variable density, the reference
    solver (not converged) and slip sides are outside the transposed step."""
    import torch
    st, g = start(name, **bad)
    grad = [torch.zeros_like(g["u"]) for _ in range(3)]
    with pytest.raises(L.LesterError):
        S.adjoint_run(g, 2, *grad)
    with pytest.raises(L.LesterError):
        S.tangent_run(g, 2, *grad)


def test_bad_configuration_refused(finalize):
    import torch
    st, g = start("box_wall")
    grad = [torch.zeros_like(g["u"]) for _ in range(3)]
    for kw in (dict(j_first=0), dict(j_first=3, j_last=2), dict(j_last=5), dict(checkpoint=0)):
        with pytest.raises(L.LesterError):
            S.adjoint_run(g, 4, *grad, **kw)
    with pytest.raises(L.LesterError):
        S.adjoint_run(g.to("numpy"), 2, *grad)


def channel_state(shape=(128, 96, 64), beta=2.2, re_tau=180.0, sigma=0.1, seed=4, cfl=0.3, model=0):
    """Stretched channel: laminar profile u = 1 - y^2 (laminar friction
    Reynolds number sqrt(2 / visc) = re_tau) plus N(0, sigma^2) noise on
    u, v, w; dt from the initial CFL number (cflest-style: max over cells
    of |u|/dx + |v|/dy + |w|/dz).  Returns (case, ctrl, device state
    after one ordinary step)."""
    import torch
    from fortranutils_gb300 import grid
    case = grid.box_case(*shape, ybc=L.BCT_WALL, beta=beta)
    s = S.new_state(case, {n: np.zeros(case.n2) for n in L.METRIC_NAMES}, np.zeros(case.n1k),
                    np.zeros(case.n1k))
    S.init_channel(s, seed=seed, sigma=sigma)
    x, y, z = case.coordinates()
    b = case.blocks[0]
    dx = np.diff(b.x[1:b.n[0]]).min()
    dy = np.diff(b.y[1:b.n[1]])
    dz = np.diff(b.z[1:b.n[2]]).min()
    u, v, w = (case.block_view(s[n], 0)[1:-1, 1:-1, 1:-1] for n in "uvw")
    c = np.abs(u) / dx + np.abs(v) / dy[None, :, None] + np.abs(w) / dz
    ctrl = L.default_ctrl(dtime=cfl / c.max(), model=model, psolve=L.PSOLVE_FP64, rtol=1e-12, max_outer=400,
                          visc=2.0 / re_tau ** 2)
    L.gpu_init(case.geom(), ctrl)
    g = s.to("torch")
    xt, yt, zt = (torch.from_numpy(a).cuda() for a in (x, y, z))
    L.comp_metric(xt, yt, zt, g["metric"], g["dkp"], g["dkw"])
    for n in ("u", "v", "w"):
        L.swap_sc(0, 1, g[n], mg_or_sg=2)
    assert S.step(g, 1) == 0
    return case, ctrl, g


@pytest.mark.parametrize("model,ndir", [(0, 16), (1, 8)])
def test_channel_gradient_against_fd_and_tangent(model, ndir, finalize):
    """128x96x64 stretched channel (tanh beta 2.2, periodic x/z), 40 steps,
    J over steps 21-40, FP64 solve, checkpoints every 10 steps, without an
    eddy-viscosity model and with Smagorinsky: the adjoint gradient against
    the tangent and against central differences along 16 (8) seeded
    directions from seed 400; the finite-difference step is picked by a
    sweep on the first direction."""
    import time
    import torch
    case, ctrl, g = channel_state(model=model)
    if model == 1:  # Smagorinsky's gam reaches a fifth of the molecular viscosity
        assert g["gam"].abs().max().item() > 0.2 * ctrl.visc
    nst, j0, j1 = 40, 21, 40
    grad = [torch.zeros_like(g["u"]) for _ in range(3)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J = S.adjoint_run(g, nst, *grad, j_first=j0, j_last=j1, checkpoint=10)
    t_adj = time.perf_counter() - t0
    zero = [torch.zeros_like(g["u"]) for _ in range(3)]

    def J_at(f):
        L.gpu_set_body_force(*f)
        try:
            return S.tangent_run(g, nst, *zero, j_first=j0, j_last=j1)[0]
        finally:
            L.gpu_set_body_force()

    def dirn(seed):
        rng = np.random.default_rng(seed)
        out = []
        for _ in range(3):
            a = np.zeros(case.n3_sg)
            v = case.block_view(a, 0)
            v[1:-1, 1:-1, 1:-1] = rng.standard_normal(v[1:-1, 1:-1, 1:-1].shape)
            out.append(torch.from_numpy(a).cuda())
        return out

    worst_tlm = worst_fd = 0.0
    eps_best = None
    for seed in range(400, 400 + ndir):
        d = dirn(seed)
        Jt, dJ = S.tangent_run(g, nst, *d, j_first=j0, j_last=j1)
        assert abs(Jt - J) <= 1e-12 * abs(J)
        adj = dot(grad, d)
        worst_tlm = max(worst_tlm, abs(adj - dJ) / abs(dJ))
        if eps_best is None:
            errs = {}
            for eps in (1e-1, 1e-2, 1e-3, 1e-4, 1e-5):
                fd = (J_at([eps * x for x in d]) - J_at([-eps * x for x in d])) / (2 * eps)
                errs[eps] = abs(fd - dJ) / abs(dJ)
            eps_best = min(errs, key=errs.get)
            print(f"\nFD step sweep (relative error vs tangent): {errs}")
        fd = (J_at([eps_best * x for x in d]) - J_at([-eps_best * x for x in d])) / (2 * eps_best)
        worst_fd = max(worst_fd, abs(fd - dJ) / abs(dJ))
    print(f"channel 128x96x64, model {model}, 40 steps, dt {ctrl.dtime:.3e}: J = {J:.10e}, adjoint run "
          f"{t_adj:.2f} s; {ndir} directions: max rel |<grad,d> - dJ_tlm| = {worst_tlm:.2e}, max rel |FD - "
          f"dJ_tlm| = {worst_fd:.2e} (eps {eps_best:g})")
    assert worst_tlm <= 1e-9
    assert worst_fd <= 1e-4
