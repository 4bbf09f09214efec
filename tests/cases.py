"""Small seeded cases shared by the tests (sizes the oracle finishes in
well under a second)."""
from __future__ import annotations

import numpy as np

from fortranutils_gb300 import grid
from fortranutils_gb300 import lester as L

import oracle_lib as O

CASES = {
    # one block, x/z periodic, y walls (the channel layout), 3 levels
    "box_wall": lambda: grid.box_case(16, 8, 12, ybc=L.BCT_WALL),
    # one block, y slip walls with tanh stretching (mixing-layer layout)
    "box_slip_stretched": lambda: grid.box_case(16, 12, 8, ybc=L.BCT_ZERO_GRAD, beta=2.0),
    # ragged: odd sizes, so no coarser level exists (single-level solve)
    "box_ragged": lambda: grid.box_case(13, 7, 9, ybc=L.BCT_WALL),
    # two uneven blocks joined by interfaces
    "two_block": lambda: grid.two_block_case(12, 8, 8, 6),
}


def metrics_dict(met) -> dict:
    return {n: np.ascontiguousarray(met[i]) for i, n in enumerate(L.METRIC_NAMES)}


class Setup:
    """Case + oracle + oracle metrics and coefficients."""

    def __init__(self, name: str, seed: int = 0):
        self.name = name
        self.case = CASES[name]()
        self.orc = O.Oracle(self.case)
        self.x, self.y, self.z = self.case.coordinates()
        met, self.dkp, self.dkw = self.orc.comp_metric(self.x, self.y, self.z)
        self.met = met
        self.m = metrics_dict(met)
        self.a = [np.zeros(self.case.n3_mg) for _ in range(7)]
        self.orc.coeff_p(self.m, self.dkp, self.dkw, self.a)
        self.rng = np.random.default_rng(seed)

    def interior_random(self, mg: bool = False, zero_mean: bool = False, scale: float = 1.0,
                        ghosts: bool = False):
        c = self.case
        f = np.zeros(c.n3_mg if mg else c.n3_sg)
        for ib in range(len(c.blocks)):
            v = c.block_view(f, ib, 0)
            if ghosts:
                v[...] = scale * self.rng.standard_normal(v.shape)
            else:
                v[1:-1, 1:-1, 1:-1] = scale * self.rng.standard_normal(v[1:-1, 1:-1, 1:-1].shape)
        if zero_mean:
            tot, cnt = 0.0, 0
            for ib in range(len(c.blocks)):
                v = c.block_view(f, ib, 0)[1:-1, 1:-1, 1:-1]
                tot += v.sum()
                cnt += v.size
            for ib in range(len(c.blocks)):
                c.block_view(f, ib, 0)[1:-1, 1:-1, 1:-1] -= tot / cnt
        return f

    def positive(self, lo=0.8, hi=1.2):
        c = self.case
        return self.rng.uniform(lo, hi, c.n3_sg)


def ctrl_for(setup: Setup, **kw):
    return L.default_ctrl(**kw)
