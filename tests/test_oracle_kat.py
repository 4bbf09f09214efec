"""Known-answer checks of the CPU oracle (no GPU).

The reference ships no tests, fixtures or golden output and cannot be built
here, so the oracle is pinned by properties that the reference algorithm
has by construction:
  * metrics of a uniform Cartesian grid are the spacings and their products;
  * coeff_p is symmetric (aw(i) = ae(i-1) ...) with zero row sums;
  * restriction sums the 8 children, prolongation reproduces constants;
  * swap_sc on a periodic box copies the opposite interior plane;
  * the multigrid solve of a manufactured compatible problem converges;
  * a uniform flow in a triply periodic box is kept by the predictor,
    except where the reference's zero metric corners act;
  * the projection leaves face mass fluxes that the pressure source sees as
    divergence free to the solver's residual.
"""
import numpy as np
import pytest

from fortranutils_gb300 import grid
from fortranutils_gb300 import lester as L
from fortranutils_gb300 import state as S

import cases
import oracle_lib as O


def interior(case, f, ib=0, lev=0):
    return case.block_view(f, ib, lev)[1:-1, 1:-1, 1:-1]


def test_uniform_grid_metrics():
    case = grid.box_case(8, 6, 4, lx=4.0, ly=3.0, lz=2.0, ybc=L.BCT_WALL)
    orc = O.Oracle(case)
    met, dkp, dkw = orc.comp_metric(*case.coordinates())
    m = cases.metrics_dict(met)
    nip1, njp1, _ = case.levels[0][0]
    o2 = case.off2[0][0]
    dip = m["dip"][o2:o2 + nip1 * njp1].reshape(njp1, nip1)
    djp = m["djp"][o2:o2 + nip1 * njp1].reshape(njp1, nip1)
    np.testing.assert_allclose(dip[1:-1, 1:-1], 0.5, rtol=1e-14)
    np.testing.assert_allclose(djp[1:-1, 1:-1], 0.5, rtol=1e-14)
    np.testing.assert_allclose(dkp[case.off1k[0][0] + 1:case.off1k[0][0] + 5], 0.5, rtol=1e-14)


@pytest.mark.parametrize("name", list(cases.CASES))
def test_coeff_p_symmetric_with_zero_row_sums(name):
    st = cases.Setup(name)
    c = st.case
    ap, aw, ae, as_, an, al, ar = st.a
    for lev in range(c.nummgl):
        for ib in range(len(c.blocks)):
            v = lambda a: c.block_view(a, ib, lev)  # noqa: E731
            P, W, E, Sa, N, Lo, R = map(v, (ap, aw, ae, as_, an, al, ar))
            it = (slice(1, -1),) * 3
            np.testing.assert_allclose(P[it], (W + E + Sa + N + Lo + R)[it], rtol=1e-12)
            # pairing of neighbouring interior points
            np.testing.assert_allclose(W[1:-1, 1:-1, 2:-1], E[1:-1, 1:-1, 1:-2], rtol=1e-12)
            np.testing.assert_allclose(Sa[1:-1, 2:-1, 1:-1], N[1:-1, 1:-2, 1:-1], rtol=1e-12)
            np.testing.assert_allclose(Lo[2:-1, 1:-1, 1:-1], R[1:-2, 1:-1, 1:-1], rtol=1e-12)
            assert np.all(P[it] > 0)


def test_restriction_sums_children_and_prolongation_keeps_constants():
    st = cases.Setup("box_wall")
    c = st.case
    f = np.zeros(c.n3_mg)
    interior(c, f)[...] = 1.5
    f1 = np.zeros(c.n3_mg)
    st.orc.restriction(2, f, f1)
    np.testing.assert_allclose(interior(c, f1, lev=1), 8 * 1.5, rtol=1e-14)
    g = np.zeros(c.n3_mg)
    c.block_view(g, 0, 1)[...] = 0.25
    st.orc.prolongation(1, g)
    np.testing.assert_allclose(interior(c, g), 0.25, rtol=1e-14)


def test_swap_sc_periodic_copies_opposite_plane():
    st = cases.Setup("box_wall", seed=3)
    c = st.case
    f = st.interior_random()
    st.orc.swap_sc(1, f, 2)
    v = c.block_view(f, 0)
    np.testing.assert_array_equal(v[1:-1, 1:-1, 0], v[1:-1, 1:-1, -2])
    np.testing.assert_array_equal(v[1:-1, 1:-1, -1], v[1:-1, 1:-1, 1])
    np.testing.assert_array_equal(v[0, 1:-1, 1:-1], v[-2, 1:-1, 1:-1])


@pytest.mark.parametrize("name", ["box_wall", "box_slip_stretched", "two_block"])
def test_lmg_solve_manufactured_problem(name):
    """b = A x for a known x: V-cycles drive ||b - A p|| / ||b|| down and
    recover x up to its (arbitrary) constant."""
    st = cases.Setup(name, seed=4)
    c = st.case
    x = st.interior_random(mg=True)
    st.orc.swap_sc(1, x, 1)
    b = np.zeros(c.n3_mg)
    res = np.zeros(c.n3_mg)
    st.orc.set_loop_bound(L.SV_P)
    # b := A x through the residual of a zero right-hand side: res = 0 - A x
    st.orc.norms(1, 1, st.a, x, b, res)
    b = -res
    for ib in range(len(c.blocks)):
        v = c.block_view(b, ib)
        keep = v[1:-1, 1:-1, 1:-1].copy()
        v[...] = 0
        v[1:-1, 1:-1, 1:-1] = keep
    p = np.zeros(c.n3_mg)
    out = st.orc.lmg_solve(O.mgctrl(nummgits=60, tolf=0.0), st.a, p, b.copy(), res)
    assert out[0] / out[1] < 1e-9, out
    d = np.concatenate([interior(c, p, ib).ravel() - interior(c, x, ib).ravel()
                        for ib in range(len(c.blocks))])
    assert np.std(d) < 1e-7 * np.std(np.concatenate(
        [interior(c, x, ib).ravel() for ib in range(len(c.blocks))]))


def test_uniform_flow_predictor():
    """Triply periodic box, uniform u = 0.7, Smagorinsky: the predicted
    velocity keeps u_int = 0.7 and w_int = 0 exactly, and v_int = 0 except
    on the edge i = ni, j = 2 of every k-plane.  There the v predictor reads
    the corner ghost (i = nip1, j = 1) of the 2-D metrics, which the
    reference leaves at zero: metric_block2.F:136-141 clamps i+1 to nip1
    (so dip(nip1, j) = 0) and the periodic metric swaps fill face ghosts
    only, not corners."""
    case = grid.box_case(8, 8, 8, ybc=L.BCT_PERIODIC)
    orc = O.Oracle(case)
    met, dkp, dkw = orc.comp_metric(*case.coordinates())
    s = S.new_state(case, cases.metrics_dict(met), dkp, dkw)
    s["u"][:] = 0.7
    for n in ("rho", "rhonp1", "rhonm1", "vd_damping"):
        s[n][:] = 1.0
    ctrl = L.default_ctrl(dtime=0.01, model=1)
    orc.step(O.mgctrl_from_ctrl(ctrl), O.phys_from_ctrl(ctrl), 1, 2, s)
    assert np.all(interior(case, s["u_int"]) == 0.7)
    assert np.all(interior(case, s["w_int"]) == 0.0)
    assert np.all(interior(case, s["gam"]) == 0.0)
    vi = interior(case, s["v_int"])
    edge = np.zeros(vi.shape, bool)
    edge[:, 0, -1] = True
    assert np.all(vi[~edge] == 0.0)
    assert np.all(vi[edge] != 0.0)
    dip = cases.metrics_dict(met)["dip"][:100].reshape(10, 10)
    assert dip[0, 9] == 0.0 and dip[9, 9] == 0.0 and dip[5, 9] > 0


def test_projection_removes_divergence():
    """After a step with a converged solve, the pressure source of the new
    velocity (its discrete divergence) is tiny next to that of the
    predicted velocity."""
    st = cases.Setup("box_wall")
    c = st.case
    s = S.init_channel(S.new_state(c, st.m, st.dkp, st.dkw), seed=5)
    ctrl = L.default_ctrl(dtime=2e-3, model=1)
    st.orc.step(O.mgctrl(nummgits=200, tolf=1e-15), O.phys_from_ctrl(ctrl), 1, 2, s)

    def source(u, v, w):
        outs = [np.zeros(c.n3_sg) for _ in range(4)]
        st.orc.sour_p(ctrl.dtime, st.m, st.dkp, st.dkw, u, v, w, s["rho"], s["rho"], outs)
        return interior(c, outs[1])

    before = source(s["u_int"], s["v_int"], s["w_int"])
    after = source(s["u"], s["v"], s["w"])
    assert np.abs(after).max() < 1e-8 * np.abs(before).max()
