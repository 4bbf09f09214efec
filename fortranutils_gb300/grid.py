"""Block layouts, grid coordinates and seeded synthetic fields.

A case is a list of blocks (points per axis including one ghost layer per
side, boundary types, neighbour links) as in the reference's block.dat, plus
vertex coordinates for every multigrid level built the way the reference
builds them:
  * level 1: interior vertices 2..nip1 from the grid, ghost vertices by
    linear extrapolation (code/xyz_extrap0.F:8-58);
  * coarser levels: every other fine vertex, x_c(i) = x_f(2i-2)
    (code/mg_xyz.F:60-120), then the same extrapolation.
Inputs are synthetic and seeded (numpy default_rng); no reference input deck
or grid file is read.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import lester as L


@dataclass
class Block:
    n: tuple            # (nip1, njp1, nkp1) points including ghosts
    bc: list            # six boundary types W E S N L R
    link: list          # six (block, side) partners, (0, 0) for none
    x: np.ndarray | None = None  # vertex coordinates along i (length nip1 + 1)
    y: np.ndarray | None = None
    z: np.ndarray | None = None
    # general 2-D interior vertices x(i, j), y(i, j), i = 2..nip1, j = 2..njp1,
    # stored (j, i) (an x.bin / y.bin block); used instead of x, y when set
    xv: np.ndarray | None = None
    yv: np.ndarray | None = None


@dataclass
class Case:
    blocks: list
    maxmgl: int = 16
    nummgl: int = 0
    gotrad: int = 0
    levels: list = field(default_factory=list)     # per level: list of (nip1, njp1, nkp1)
    off3: list = field(default_factory=list)
    off2: list = field(default_factory=list)
    off1k: list = field(default_factory=list)
    offxy: list = field(default_factory=list)
    offz: list = field(default_factory=list)

    # -------------------------------------------------------- geometry
    def setup(self) -> "Case":
        """Level search and offsets (code/set_offset.F:94-234)."""
        dims = [[tuple(b.n) for b in self.blocks]]
        found = 1
        for lev in range(1, self.maxmgl):
            nxt, ok = [], True
            for n in dims[-1]:
                if all(v % 2 == 0 for v in n) and all(v // 2 + 1 >= 4 for v in n):
                    nxt.append(tuple(v // 2 + 1 for v in n))
                else:
                    ok = False
                    break
            if not ok:
                break
            dims.append(nxt)
            found = lev + 1
        self.nummgl = found if self.nummgl == 0 else self.nummgl
        if self.nummgl > found:
            raise ValueError(f"levels found {found}, required {self.nummgl}")
        self.levels = dims[: self.nummgl]
        o3 = o2 = o1 = oxy = oz = 0
        self.off3, self.off2, self.off1k, self.offxy, self.offz = [], [], [], [], []
        for lev in self.levels:
            r3, r2, r1, rxy, rz = [], [], [], [], []
            for (a, b, c) in lev:
                r3.append(o3); r2.append(o2); r1.append(o1); rxy.append(oxy); rz.append(oz)
                o3 += a * b * c; o2 += a * b; o1 += c; oxy += (a + 1) * (b + 1); oz += c + 1
            self.off3.append(r3); self.off2.append(r2); self.off1k.append(r1)
            self.offxy.append(rxy); self.offz.append(rz)
        self.n3_mg, self.n2, self.n1k, self.nxy, self.nz = o3, o2, o1, oxy, oz
        self.n3_sg = sum(a * b * c for (a, b, c) in self.levels[0])
        return self

    def geom(self) -> L.Geom:
        g = L.Geom()
        g.numbl = len(self.blocks)
        g.maxmgl = self.maxmgl
        g.nummgl = self.nummgl
        g.gotrad = self.gotrad
        for ib, b in enumerate(self.blocks):
            for d in range(3):
                g.bl_nijkp1[ib][d] = b.n[d]
            for s in range(6):
                g.bl_bc[ib][s] = b.bc[s]
                g.bl2bl[ib][s] = b.link[s][0]
                g.bl2side[ib][s] = b.link[s][1]
        return g

    def oracle_args(self):
        """(numbl, nijkp1, bc, bl2bl, bl2side) as flat int32 arrays."""
        nb = len(self.blocks)
        n = np.array([b.n for b in self.blocks], dtype=np.int32).ravel()
        bc = np.array([b.bc for b in self.blocks], dtype=np.int32).ravel()
        l1 = np.array([[s[0] for s in b.link] for b in self.blocks], dtype=np.int32).ravel()
        l2 = np.array([[s[1] for s in b.link] for b in self.blocks], dtype=np.int32).ravel()
        return nb, n, bc, l1, l2

    # ------------------------------------------------------- coordinates
    def coordinates(self):
        """x, y (2-D vertex arrays) and z for every level, flat, mg layout."""
        x = np.zeros(self.nxy)
        y = np.zeros(self.nxy)
        z = np.zeros(self.nz)
        fine = []
        for ib, b in enumerate(self.blocks):
            nip1, njp1, nkp1 = b.n
            nip2, njp2, nkp2 = nip1 + 1, njp1 + 1, nkp1 + 1
            X = np.zeros((njp2, nip2))
            Y = np.zeros((njp2, nip2))
            if b.xv is not None:
                X[1:njp1, 1:nip1] = b.xv
                Y[1:njp1, 1:nip1] = b.yv
            else:
                X[1:njp1, 1:nip1] = b.x[None, 1:nip1]
                Y[1:njp1, 1:nip1] = b.y[1:njp1, None]
            Z = np.zeros(nkp2)
            Z[1:nkp1] = b.z[1:nkp1]
            _extrap2(X)
            _extrap2(Y)
            _extrap1(Z)
            fine.append((X, Y, Z))
        for lev in range(self.nummgl):
            for ib, (nip1, njp1, nkp1) in enumerate(self.levels[lev]):
                nip2, njp2, nkp2 = nip1 + 1, njp1 + 1, nkp1 + 1
                if lev == 0:
                    X, Y, Z = fine[ib]
                else:
                    Xf, Yf, Zf = prev[ib]
                    X = np.zeros((njp2, nip2))
                    Y = np.zeros((njp2, nip2))
                    Z = np.zeros(nkp2)
                    # x_c(i_c, j_c) = x_f(2 i_c - 2, 2 j_c - 2), i_c = 2..nip2_c - 1
                    ic = np.arange(2, nip2)
                    jc = np.arange(2, njp2)
                    X[np.ix_(jc - 1, ic - 1)] = Xf[np.ix_(2 * jc - 3, 2 * ic - 3)]
                    Y[np.ix_(jc - 1, ic - 1)] = Yf[np.ix_(2 * jc - 3, 2 * ic - 3)]
                    kc = np.arange(2, nkp2)
                    Z[kc - 1] = Zf[2 * kc - 3]
                    _extrap2(X)
                    _extrap2(Y)
                    _extrap1(Z)
                    fine[ib] = (X, Y, Z)
                o = self.offxy[lev][ib]
                x[o:o + X.size] = X.ravel()
                y[o:o + Y.size] = Y.ravel()
                oz = self.offz[lev][ib]
                z[oz:oz + Z.size] = Z
            prev = list(fine)
        return x, y, z

    def field3(self, mg: bool = False) -> np.ndarray:
        return np.zeros(self.n3_mg if mg else self.n3_sg)

    def block_view(self, a: np.ndarray, ib: int, lev: int = 0) -> np.ndarray:
        """(k, j, i) view of block ib (0-based) at level lev of a 3-D field."""
        nip1, njp1, nkp1 = self.levels[lev][ib]
        o = self.off3[lev][ib]
        return a[o:o + nip1 * njp1 * nkp1].reshape(nkp1, njp1, nip1)

    def cells(self) -> int:
        return sum((a - 2) * (b - 2) * (c - 2) for (a, b, c) in self.levels[0])


def _extrap2(X):
    """code/xyz_extrap0.F:36-50 (array stored (j, i))."""
    X[:, 0] = 2.0 * X[:, 1] - X[:, 2]
    X[:, -1] = 2.0 * X[:, -2] - X[:, -3]
    X[0, :] = 2.0 * X[1, :] - X[2, :]
    X[-1, :] = 2.0 * X[-2, :] - X[-3, :]


def _extrap1(Z):
    Z[0] = 2.0 * Z[1] - Z[2]
    Z[-1] = 2.0 * Z[-2] - Z[-3]


def _axis(n_int: int, lo: float, hi: float, beta: float | None = None) -> np.ndarray:
    """Vertex coordinates 1..n+3 (index 0..n+2): interior vertices at 1..n+1."""
    eta = np.linspace(-1.0, 1.0, n_int + 1)
    if beta:
        s = np.tanh(beta * eta) / np.tanh(beta)
    else:
        s = eta
    v = lo + (s + 1.0) * 0.5 * (hi - lo)
    out = np.zeros(n_int + 3)
    out[1:n_int + 2] = v
    return out


def box_case(ni: int, nj: int, nk: int, lx: float = 2 * np.pi, ly: float = 2.0,
             lz: float = np.pi, ybc: int = L.BCT_WALL, xbc: int = L.BCT_PERIODIC,
             zbc: int = L.BCT_PERIODIC, beta: float | None = None, maxmgl: int = 16,
             nummgl: int = 0) -> Case:
    """One block of ni x nj x nk cells on [0,lx] x [-ly/2, ly/2] x [0,lz]."""
    bc = [xbc, xbc, ybc, ybc, zbc, zbc]
    link = [(0, 0)] * 6
    for ax, t in enumerate((xbc, ybc, zbc)):
        if t == L.BCT_PERIODIC:
            link[2 * ax] = (1, 2 * ax + 2)
            link[2 * ax + 1] = (1, 2 * ax + 1)
    b = Block(n=(ni + 2, nj + 2, nk + 2), bc=bc, link=link,
              x=_axis(ni, 0.0, lx), y=_axis(nj, -ly / 2, ly / 2, beta), z=_axis(nk, 0.0, lz))
    return Case(blocks=[b], maxmgl=maxmgl, nummgl=nummgl).setup()


def two_block_case(ni1: int, ni2: int, nj: int, nk: int, ybc: int = L.BCT_WALL,
                   maxmgl: int = 16, nummgl: int = 0) -> Case:
    """Two blocks side by side in x joined by an interface, periodic in x
    across the pair and in z: block 1 east <-> block 2 west (interface),
    block 2 east <-> block 1 west (interface, closing the period)."""
    lx = 2.0 * np.pi
    xs = _axis(ni1 + ni2, 0.0, lx)
    x1 = np.zeros(ni1 + 3)
    x1[1:ni1 + 2] = xs[1:ni1 + 2]
    x2 = np.zeros(ni2 + 3)
    x2[1:ni2 + 2] = xs[ni1 + 1:ni1 + ni2 + 2]
    yv = _axis(nj, -1.0, 1.0)
    zv = _axis(nk, 0.0, np.pi)
    I, P = L.BCT_INTERFACE, L.BCT_PERIODIC
    b1 = Block(n=(ni1 + 2, nj + 2, nk + 2), bc=[I, I, ybc, ybc, P, P],
               link=[(2, 2), (2, 1), (0, 0), (0, 0), (1, 6), (1, 5)], x=x1, y=yv, z=zv)
    b2 = Block(n=(ni2 + 2, nj + 2, nk + 2), bc=[I, I, ybc, ybc, P, P],
               link=[(1, 2), (1, 1), (0, 0), (0, 0), (2, 6), (2, 5)], x=x2, y=yv, z=zv)
    return Case(blocks=[b1, b2], maxmgl=maxmgl, nummgl=nummgl).setup()


def boxes_case(sizes, ybc: int = L.BCT_WALL, h: float | None = None, maxmgl: int = 16,
               nummgl: int = 0) -> Case:
    """Independent boxes, one block each: (ni, nj, nk) cells, each periodic
    in x and z onto itself and bounded in y by `ybc` sides, on
    [0, 2 pi] x [-1, 1] x [0, pi], or with cubic cells of side h on
    [0, ni h] x [-nj h / 2, nj h / 2] x [0, nk h].  No block links to
    another, so a singular pressure operator has one constant null vector
    per box."""
    blocks = []
    for ib, (ni, nj, nk) in enumerate(sizes, start=1):
        link = [(ib, 2), (ib, 1), (0, 0), (0, 0), (ib, 6), (ib, 5)]
        P = L.BCT_PERIODIC
        lx, ly, lz = (2 * np.pi, 2.0, np.pi) if h is None else (ni * h, nj * h, nk * h)
        blocks.append(Block(n=(ni + 2, nj + 2, nk + 2), bc=[P, P, ybc, ybc, P, P], link=link,
                            x=_axis(ni, 0.0, lx), y=_axis(nj, -ly / 2, ly / 2), z=_axis(nk, 0.0, lz)))
    return Case(blocks=blocks, maxmgl=maxmgl, nummgl=nummgl).setup()


def inflow_case(ni1: int, ni2: int, nj: int, nk: int, ybc: int = L.BCT_WALL, beta: float | None = None,
                maxmgl: int = 16, nummgl: int = 0) -> Case:
    """A spatially developing channel of two blocks in x joined by an
    interface: block 1's west side a fixed inflow (BCT_FIXED), block 2's
    east side a convective outflow (BCT_CONVECTIVE), `ybc` sides in y,
    periodic in z."""
    lx = 4.0 * np.pi
    xs = _axis(ni1 + ni2, 0.0, lx)
    x1 = np.zeros(ni1 + 3)
    x1[1:ni1 + 2] = xs[1:ni1 + 2]
    x2 = np.zeros(ni2 + 3)
    x2[1:ni2 + 2] = xs[ni1 + 1:ni1 + ni2 + 2]
    yv = _axis(nj, -1.0, 1.0, beta)
    zv = _axis(nk, 0.0, np.pi)
    I, P, F, Cv = L.BCT_INTERFACE, L.BCT_PERIODIC, L.BCT_FIXED, L.BCT_CONVECTIVE
    b1 = Block(n=(ni1 + 2, nj + 2, nk + 2), bc=[F, I, ybc, ybc, P, P],
               link=[(0, 0), (2, 1), (0, 0), (0, 0), (1, 6), (1, 5)], x=x1, y=yv, z=zv)
    b2 = Block(n=(ni2 + 2, nj + 2, nk + 2), bc=[I, Cv, ybc, ybc, P, P],
               link=[(1, 2), (0, 0), (0, 0), (0, 0), (2, 6), (2, 5)], x=x2, y=yv, z=zv)
    return Case(blocks=[b1, b2], maxmgl=maxmgl, nummgl=nummgl).setup()


BL6_LOWER = ((160, 96, 64), (128, 96, 64), (96, 96, 64))
BL6_UPPER = ((160, 48, 64), (128, 48, 64), (96, 48, 64))


def bl6_case(div: int = 1, maxmgl: int = 16, nummgl: int = 0) -> Case:
    """Multiblock boundary layer: two rows of three blocks of uneven sizes
    (cells, divided by `div`): lower (160,96,64) (128,96,64) (96,96,64) on
    y in [0, 2], upper (160,48,64) (128,48,64) (96,48,64) on y in [2, 3],
    joined by interfaces in x and y; x = 0 a fixed inflow (blocks 1 and 4),
    the east end a convective outflow (blocks 3 and 6), a wall at y = 0, a
    slip side at y = 3, periodic in z (depth 2).  Cubic cells of side
    1/32 (times div)."""
    lo = [tuple(v // div for v in s) for s in BL6_LOWER]
    up = [tuple(v // div for v in s) for s in BL6_UPPER]
    h = div / 32.0
    I, P, F, Cv, W, Z = (L.BCT_INTERFACE, L.BCT_PERIODIC, L.BCT_FIXED, L.BCT_CONVECTIVE, L.BCT_WALL,
                         L.BCT_ZERO_GRAD)
    nx = [s[0] for s in lo]
    x0 = np.cumsum([0] + nx) * h
    blocks = []
    for row, sizes in enumerate((lo, up)):
        for col, (ni, nj, nk) in enumerate(sizes):
            b = 3 * row + col + 1
            bc = [F if col == 0 else I, Cv if col == 2 else I, W if row == 0 else I, Z if row == 1 else I, P, P]
            link = [(0, 0) if col == 0 else (b - 1, 2), (0, 0) if col == 2 else (b + 1, 1),
                    (0, 0) if row == 0 else (b - 3, 4), (0, 0) if row == 1 else (b + 3, 3), (b, 6), (b, 5)]
            y0, y1 = (0.0, 2.0) if row == 0 else (2.0, 3.0)
            blocks.append(Block(n=(ni + 2, nj + 2, nk + 2), bc=bc, link=link, x=_axis(ni, x0[col], x0[col + 1]),
                                y=_axis(nj, y0, y1), z=_axis(nk, 0.0, nk * h)))
    return Case(blocks=blocks, maxmgl=maxmgl, nummgl=nummgl).setup()


def bl6_inflow(case, delta: float = 0.5, uinf: float = 1.0):
    """u, v inflow profiles of the bl6 case for inlet slots 1 (block 1) and
    4 (block 4) of fixed_inlet: u = uinf tanh(y / delta) at the cell
    centres (ghosts included) of each inlet block, v = 0."""
    b1, b4 = case.blocks[0], case.blocks[3]
    nj4 = b4.n[1] - 1
    off4 = 3 * (nj4 - 1)
    n = max(b1.n[1], off4 + b4.n[1], 4 * (nj4 - 2)) + 1
    up, vp = np.zeros(n), np.zeros(n)
    for b, off in ((b1, 0), (b4, off4)):
        yc = 0.5 * (b.y[:-1] + b.y[1:])[: b.n[1]]
        up[off:off + b.n[1]] = uinf * np.tanh(np.maximum(yc, 0.0) / delta)
    return np.ascontiguousarray(up), np.ascontiguousarray(vp)


def chain_case(nblocks: int, ni: int, nj: int, nk: int, ybc: int = L.BCT_WALL) -> Case:
    """`nblocks` equal blocks in a row along x joined by interfaces: a fixed
    inflow on block 1's west side, a convective outflow on the last block's
    east side, `ybc` sides in y, periodic in z (a recycling chain)."""
    I, P, F, Cv = L.BCT_INTERFACE, L.BCT_PERIODIC, L.BCT_FIXED, L.BCT_CONVECTIVE
    lx = 0.5 * nblocks
    xs = _axis(ni * nblocks, 0.0, lx)
    blocks = []
    for b in range(1, nblocks + 1):
        x = np.zeros(ni + 3)
        x[1:ni + 2] = xs[(b - 1) * ni + 1:b * ni + 2]
        bc = [F if b == 1 else I, Cv if b == nblocks else I, ybc, ybc, P, P]
        link = [(0, 0) if b == 1 else (b - 1, 2), (0, 0) if b == nblocks else (b + 1, 1), (0, 0), (0, 0),
                (b, 6), (b, 5)]
        blocks.append(Block(n=(ni + 2, nj + 2, nk + 2), bc=bc, link=link, x=x, y=_axis(nj, -1.0, 1.0),
                            z=_axis(nk, 0.0, 1.0)))
    return Case(blocks=blocks).setup()
