"""Deck and dump formats of the reference (fortranutils_gb300.lesio):
block.dat and x/y/z.bin round trips into a case equal to the generated
one, Fortran sequential unformatted dumps (REAL*4 and REAL*8) checked
byte by byte against the record layout of code/file_3.F, and the
formatted dumps.  CPU only."""
import struct

import numpy as np
import pytest

from fortranutils_gb300 import grid, lesio
from fortranutils_gb300 import lester as L


def test_deck_round_trip(tmp_path):
    case = grid.bl6_case(8)
    lesio.write_deck(tmp_path, case)
    back = lesio.case_from_deck(tmp_path)
    assert back.levels == case.levels
    g0, g1 = case.geom(), back.geom()
    for ib in range(len(case.blocks)):
        assert list(g0.bl_bc[ib]) == list(g1.bl_bc[ib])
        assert list(g0.bl2bl[ib]) == list(g1.bl2bl[ib])
        assert list(g0.bl2side[ib]) == list(g1.bl2side[ib])
    for a, b in zip(case.coordinates(), back.coordinates()):
        np.testing.assert_allclose(b, a, rtol=1e-8, atol=1e-12)


def test_list_directed_reads():
    """Each read starts on a new line and takes values across lines; repeat
    counts expand; the rest of the last line is dropped."""
    r = lesio._ListReader("1 2 3 9 9\n4,5\n6 7 8\n3*2.5 1.0d0\n")
    assert r.read(3, int) == [1, 2, 3]
    assert r.read(4, int) == [4, 5, 6, 7]
    assert r.read(4) == [2.5, 2.5, 2.5, 1.0]


def _expected_binary(case, f, dt):
    out = b""

    def rec(p):
        return struct.pack("<i", len(p)) + p + struct.pack("<i", len(p))
    out += rec(struct.pack("<i", len(case.blocks)))
    for n in case.levels[0]:
        out += rec(struct.pack("<3i", *n))
    for ib, (nip1, njp1, nkp1) in enumerate(case.levels[0]):
        v = case.block_view(f, ib)
        for k in range(nkp1):
            for j in range(njp1):
                out += rec(v[k, j, :].astype(dt).tobytes())
    return out


@pytest.mark.parametrize("double", [False, True])
def test_binary_dump_layout(tmp_path, double):
    case = grid.two_block_case(6, 4, 4, 2)
    f = np.random.default_rng(3).standard_normal(case.n3_sg)
    p = tmp_path / "u.dat"
    lesio.write_dump(p, case, f, binary=True, double=double)
    assert p.read_bytes() == _expected_binary(case, f, np.float64 if double else np.float32)
    back = lesio.read_dump(p, case, binary=True, double=double)
    np.testing.assert_array_equal(back, f if double else f.astype(np.float32).astype(np.float64))


def test_formatted_dump_round_trip(tmp_path):
    case = grid.box_case(10, 4, 4)
    f = np.random.default_rng(4).standard_normal(case.n3_sg)
    p = tmp_path / "u.txt"
    lesio.write_dump(p, case, f, binary=False)
    back = lesio.read_dump(p, case, binary=False)
    np.testing.assert_allclose(back, f, rtol=1e-8)
    # eight values per line, as '(8(1x,g15.8))' writes them
    lines = p.read_text().splitlines()
    assert all(len(ln.split()) <= 8 for ln in lines[2:])


def test_dump_dimension_checks(tmp_path):
    a, b = grid.box_case(8, 4, 4), grid.box_case(8, 6, 4)
    p = tmp_path / "u.dat"
    lesio.write_dump(p, a, np.zeros(a.n3_sg))
    with pytest.raises(ValueError):
        lesio.read_dump(p, b)
    bad = bytearray(p.read_bytes())
    bad[-1] ^= 1
    p.write_bytes(bytes(bad))
    with pytest.raises(ValueError):
        lesio.read_dump(p, a)


@pytest.mark.gpu
def test_deck_drives_gpu_step(tmp_path, gpulib):
    """A case read from block.dat and x/y/z.bin runs through lester_step and
    matches the oracle on the same deck; the result dumps and reads back."""
    import cases
    import oracle_lib as O
    from fortranutils_gb300 import state as S
    lesio.write_deck(tmp_path, grid.inflow_case(12, 8, 8, 6))
    case = lesio.case_from_deck(tmp_path)
    cases.CASES["deck"] = lambda: case
    try:
        st = cases.Setup("deck", seed=2)
    finally:
        del cases.CASES["deck"]
    ctrl = L.default_ctrl(dtime=2e-3, model=1)
    s = S.new_state(case, st.m, st.dkp, st.dkw)
    S.init_channel(s, seed=9)
    ref = s.to("numpy")
    mg, k = O.mgctrl_from_ctrl(ctrl), O.phys_from_ctrl(ctrl)
    for it in (1, 2):
        st.orc.step(mg, k, it, it + 1, ref)
    L.gpu_init(case.geom(), ctrl)
    try:
        g = s.to("torch")
        for it in (1, 2):
            assert S.step(g, it) == 0
        got = g.to("numpy")
    finally:
        L.gpu_finalize()
    for n in ("u", "v", "w", "p"):
        assert np.linalg.norm(got[n] - ref[n]) <= 1e-10 * np.linalg.norm(ref[n]), n
    lesio.write_dump(tmp_path / "u.dat", case, got["u"], double=True)
    np.testing.assert_array_equal(lesio.read_dump(tmp_path / "u.dat", case, double=True), got["u"])
