"""Readers and writers of the reference's input decks and field dumps, so a
LESter case directory can drive the GPU path and its dumps can be read back.

block.dat (code/read_bl_info.F:43-130), list-directed text:
    a header line, then per block: bl2pe, (bl2bl, bl2side) x 6;
    a header line, then per block: bl_bc x 6;
    a header line, then per block: bl_split x 6.
x.bin, y.bin, z.bin (code/read_xyz.F:63-128), list-directed text:
    numbl; per block nip1 njp1 nkp1; then per block, for x and y, one record
    per j = 2..njp1 of the nip1 - 1 vertex values i = 2..nip1, and for z one
    record of the nkp1 - 1 values k = 2..nkp1.  (Ghost vertices are
    extrapolated afterwards, code/xyz_extrap0.F.)
Field dumps (code/file_3.F:80-166, read_3.F:85-134):
    unformatted (filefrmt 0): Fortran sequential records with 4-byte length
    markers -- one record int32 numbl, one record of three int32 (nip1,
    njp1, nkp1) per block, then per block, per k, per j, one record of the
    nip1 values of that row, REAL*4 (or REAL*8 when the reference is built
    with WRITE_DOUBLE / READ_DOUBLE);
    formatted: the same numbers, list-directed, the rows written
    '(8(1x,g15.8))'.  This writer uses 1PE15.8 fields in that layout (eight
    per line), which any list-directed reader, the reference's included,
    reads the same way.

Arrays are numpy, in the arena layouts of fortranutils_gb300.grid (sg or
level 1 of mg for 3-D fields).  Host-side only: nothing here touches the GPU.
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

from . import grid


# ------------------------------------------------------------- list-directed
class _ListReader:
    """Fortran list-directed reads over text lines: each read starts on a
    new line, takes values across lines until it has enough, and drops the
    rest of its last line.  `r*c` repeat counts are expanded."""

    def __init__(self, text: str):
        self.lines = text.splitlines()
        self.pos = 0

    def skip(self):
        self.pos += 1

    def read(self, n: int, conv=float):
        out = []
        while len(out) < n:
            if self.pos >= len(self.lines):
                raise ValueError(f"end of file: wanted {n} values, got {len(out)}")
            line = self.lines[self.pos].split("!")[0].replace(",", " ")
            self.pos += 1
            for tok in line.split():
                if tok == "/":
                    break
                if "*" in tok:
                    r, c = tok.split("*", 1)
                    out.extend([c] * int(r))
                else:
                    out.append(tok)
        return [conv(t.replace("d", "e").replace("D", "E")) if conv is float else conv(t) for t in out[:n]]


def _fmt_rows(values, per_line: int = 8) -> str:
    """'(8(1x,1pe15.8))'-style lines: eight values per line."""
    lines = []
    for s in range(0, len(values), per_line):
        lines.append("".join(" " + f"{v: .8E}".rjust(15) for v in values[s:s + per_line]))
    return "\n".join(lines)


# --------------------------------------------------------------- block.dat
def read_block_dat(path, numbl: int) -> dict:
    """bl2pe, bl2bl, bl2side, bl_bc (int arrays (numbl, 6) / (numbl,)) and
    bl_split (float (numbl, 6)) of code/read_bl_info.F:81-130."""
    r = _ListReader(Path(path).read_text())
    bl2pe = np.zeros(numbl, dtype=np.int32)
    bl2bl = np.zeros((numbl, 6), dtype=np.int32)
    bl2side = np.zeros((numbl, 6), dtype=np.int32)
    bl_bc = np.zeros((numbl, 6), dtype=np.int32)
    bl_split = np.zeros((numbl, 6))
    r.skip()
    for b in range(numbl):
        v = r.read(13, int)
        bl2pe[b] = v[0]
        bl2bl[b] = v[1::2]
        bl2side[b] = v[2::2]
    r.skip()
    for b in range(numbl):
        bl_bc[b] = r.read(6, int)
    r.skip()
    for b in range(numbl):
        try:
            bl_split[b] = r.read(6, float)
        except ValueError:
            break  # a deck without the split section
    return dict(bl2pe=bl2pe, bl2bl=bl2bl, bl2side=bl2side, bl_bc=bl_bc, bl_split=bl_split)


def write_block_dat(path, bl2bl, bl2side, bl_bc, bl2pe=None, bl_split=None) -> None:
    nb = len(bl_bc)
    bl2pe = np.zeros(nb, dtype=int) if bl2pe is None else bl2pe
    bl_split = np.zeros((nb, 6)) if bl_split is None else bl_split
    out = ["  pe   (block side) x 6: W E S N L R"]
    for b in range(nb):
        pairs = " ".join(f"{int(bl2bl[b][s]):4d} {int(bl2side[b][s]):2d}" for s in range(6))
        out.append(f"{int(bl2pe[b]):4d} {pairs}")
    out.append("  boundary types W E S N L R")
    for b in range(nb):
        out.append(" ".join(f"{int(t):4d}" for t in bl_bc[b]))
    out.append("  outflow split W E S N L R")
    for b in range(nb):
        out.append(" ".join(f"{float(t):.6f}" for t in bl_split[b]))
    Path(path).write_text("\n".join(out) + "\n")


# ----------------------------------------------------------- x/y/z.bin
def read_grid_file(path, kind: str):
    """(nijkp1 per block, vertex arrays per block): kind 'x' or 'y' gives
    (njp1 - 1, nip1 - 1) arrays of the vertices i = 2..nip1, j = 2..njp1;
    kind 'z' gives the nkp1 - 1 vertices k = 2..nkp1."""
    r = _ListReader(Path(path).read_text())
    nb = r.read(1, int)[0]
    dims = [tuple(r.read(3, int)) for _ in range(nb)]
    arrays = []
    for (nip1, njp1, nkp1) in dims:
        if kind == "z":
            arrays.append(np.array(r.read(nkp1 - 1)))
        else:
            arrays.append(np.array([r.read(nip1 - 1) for _ in range(2, njp1 + 1)]))
    return dims, arrays


def write_grid_file(path, dims, arrays, kind: str) -> None:
    out = [f" {len(dims)}"]
    out += [f" {a} {b} {c}" for (a, b, c) in dims]
    for (nip1, njp1, nkp1), arr in zip(dims, arrays):
        if kind == "z":
            out.append(_fmt_rows(list(arr[: nkp1 - 1])))
        else:
            for j in range(njp1 - 1):
                out.append(_fmt_rows(list(arr[j, : nip1 - 1])))
    Path(path).write_text("\n".join(out) + "\n")


def case_from_deck(directory, maxmgl: int = 16, nummgl: int = 0) -> grid.Case:
    """A grid.Case from a case directory's block.dat and x.bin, y.bin,
    z.bin (general 2-D x(i,j), y(i,j) per block)."""
    d = Path(directory)
    dims, xs = read_grid_file(d / "x.bin", "x")
    dims_y, ys = read_grid_file(d / "y.bin", "y")
    dims_z, zs = read_grid_file(d / "z.bin", "z")
    if dims != dims_y or dims != dims_z:
        raise ValueError("x.bin, y.bin and z.bin disagree on the block dimensions")
    info = read_block_dat(d / "block.dat", len(dims))
    blocks = []
    for b, n in enumerate(dims):
        link = [(int(info["bl2bl"][b][s]), int(info["bl2side"][b][s])) for s in range(6)]
        z = np.zeros(n[2] + 1)
        z[1:n[2]] = zs[b]
        blocks.append(grid.Block(n=n, bc=[int(t) for t in info["bl_bc"][b]], link=link, z=z,
                                 xv=xs[b], yv=ys[b]))
    return grid.Case(blocks=blocks, maxmgl=maxmgl, nummgl=nummgl).setup()


def write_deck(directory, case: grid.Case) -> None:
    """block.dat and x/y/z.bin of a case (level-1 interior vertices)."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    x, y, z = case.coordinates()
    dims = [tuple(b.n) for b in case.blocks]
    xs, ys, zs = [], [], []
    for ib, (nip1, njp1, nkp1) in enumerate(dims):
        o = case.offxy[0][ib]
        X = x[o:o + (nip1 + 1) * (njp1 + 1)].reshape(njp1 + 1, nip1 + 1)
        Y = y[o:o + (nip1 + 1) * (njp1 + 1)].reshape(njp1 + 1, nip1 + 1)
        xs.append(X[1:njp1, 1:nip1])
        ys.append(Y[1:njp1, 1:nip1])
        oz = case.offz[0][ib]
        zs.append(z[oz + 1:oz + nkp1])
    write_grid_file(d / "x.bin", dims, xs, "x")
    write_grid_file(d / "y.bin", dims, ys, "y")
    write_grid_file(d / "z.bin", dims, zs, "z")
    write_block_dat(d / "block.dat", [[s[0] for s in b.link] for b in case.blocks],
                    [[s[1] for s in b.link] for b in case.blocks], [b.bc for b in case.blocks])


# ------------------------------------------------------------- field dumps
def _records(buf: bytes):
    """Fortran sequential unformatted records (4-byte markers)."""
    pos = 0
    while pos < len(buf):
        (n,) = struct.unpack_from("<i", buf, pos)
        if n < 0:
            raise ValueError("subrecords (records over 2 GiB) are not supported")
        rec = buf[pos + 4:pos + 4 + n]
        (n2,) = struct.unpack_from("<i", buf, pos + 4 + n)
        if n2 != n:
            raise ValueError(f"record markers disagree at byte {pos}: {n} and {n2}")
        yield rec
        pos += 8 + n


def write_dump(path, case: grid.Case, f: np.ndarray, binary: bool = True, double: bool = False) -> None:
    """code/file_3.F: f in the level-1 (sg) layout of `case`."""
    dims = [tuple(v) for v in case.levels[0]]
    if binary:
        dt = np.float64 if double else np.float32
        parts = []

        def rec(payload: bytes):
            parts.append(struct.pack("<i", len(payload)) + payload + struct.pack("<i", len(payload)))

        rec(struct.pack("<i", len(dims)))
        for n in dims:
            rec(struct.pack("<3i", *n))
        for ib, (nip1, njp1, nkp1) in enumerate(dims):
            v = case.block_view(f, ib)
            for k in range(nkp1):
                for j in range(njp1):
                    rec(np.ascontiguousarray(v[k, j, :], dtype=dt).tobytes())
        Path(path).write_bytes(b"".join(parts))
    else:
        out = [f" {len(dims)}"] + [f" {a} {b} {c}" for (a, b, c) in dims]
        for ib, (nip1, njp1, nkp1) in enumerate(dims):
            v = case.block_view(f, ib)
            for k in range(nkp1):
                for j in range(njp1):
                    out.append(_fmt_rows(list(v[k, j, :])))
        Path(path).write_text("\n".join(out) + "\n")


def read_dump(path, case: grid.Case, binary: bool = True, double: bool = False) -> np.ndarray:
    """code/read_3.F: a dump into a new level-1 (sg) array of `case`;
    block count and dimensions are checked as read_3.F:100-128 does."""
    dims = [tuple(v) for v in case.levels[0]]
    f = np.zeros(case.n3_sg)
    if binary:
        dt = np.float64 if double else np.float32
        recs = _records(Path(path).read_bytes())
        (nb,) = struct.unpack("<i", next(recs))
        if nb != len(dims):
            raise ValueError(f"dump has {nb} blocks, the case {len(dims)}")
        for ib in range(nb):
            n = struct.unpack("<3i", next(recs))
            if tuple(n) != dims[ib]:
                raise ValueError(f"block {ib + 1}: dump {n}, case {dims[ib]}")
        for ib, (nip1, njp1, nkp1) in enumerate(dims):
            v = case.block_view(f, ib)
            for k in range(nkp1):
                for j in range(njp1):
                    row = np.frombuffer(next(recs), dtype=dt)
                    if row.size != nip1:
                        raise ValueError(f"block {ib + 1} row ({j + 1}, {k + 1}): {row.size} values")
                    v[k, j, :] = row
    else:
        r = _ListReader(Path(path).read_text())
        nb = r.read(1, int)[0]
        if nb != len(dims):
            raise ValueError(f"dump has {nb} blocks, the case {len(dims)}")
        for ib in range(nb):
            n = tuple(r.read(3, int))
            if n != dims[ib]:
                raise ValueError(f"block {ib + 1}: dump {n}, case {dims[ib]}")
        for ib, (nip1, njp1, nkp1) in enumerate(dims):
            v = case.block_view(f, ib)
            for k in range(nkp1):
                for j in range(njp1):
                    v[k, j, :] = r.read(nip1)
    return f
