"""lester_norms_noalloc, the allocation-free residual and norms of one block,
against lester_norms through the C ABI.

The entry point serves hosts that must not allocate device memory when they
call it (a fixed device-memory budget, or a host-owned pool that libraries
may not bypass).  Its arithmetic and reduction order are those of
lester_norms, so residual and norms must agree bit for bit.

Collected last (file name), so it runs both after every other test and,
alone, in a fresh process.  The allocation-free call is made before any
lester_gpu_init, so it is shown to need no library context.
"""
import ctypes as C

import numpy as np
import pytest

from fortranutils_gb300 import lester as L

import cases

pytestmark = pytest.mark.gpu


def noalloc(case, a, x, b, residu):
    import torch
    n = (C.c_int * 3)(*case.levels[0][0])
    out = [C.c_double() for _ in range(4)]
    rc = L.lib().lester_norms_noalloc(n, *[L._p(t) for t in a], L._p(x), L._p(b), L._p(residu),
                                      *[C.byref(o) for o in out],
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, [o.value for o in out]


@pytest.mark.parametrize("name", ["box_wall", "box_slip_stretched", "box_ragged"])
def test_noalloc_matches_norms_two_calls(name, gpulib):
    import torch
    st = cases.Setup(name, seed=21)
    c = st.case
    dev = lambda v: torch.from_numpy(np.ascontiguousarray(v)).cuda()  # noqa: E731
    a = [dev(t) for t in st.a]
    xs = [dev(st.interior_random(mg=True, ghosts=True)) for _ in range(2)]
    bs = [dev(st.interior_random(mg=True)) for _ in range(2)]
    L.gpu_finalize()  # no library context for the allocation-free calls
    got = []
    for x, b in zip(xs, bs):
        r = torch.full((c.n3_mg,), 7.0, dtype=torch.float64, device="cuda")
        rc, nrm = noalloc(c, a, x, b, r)
        assert rc == 0, L.lib().lester_gpu_last_error()
        got.append((nrm, r.cpu().numpy()))
    L.gpu_init(c.geom(), L.default_ctrl())
    try:
        for (nrm, r), x, b in zip(got, xs, bs):
            rr = torch.full((c.n3_mg,), 7.0, dtype=torch.float64, device="cuda")
            ref = L.norms(1, 1, *a, x, b, rr)
            # same FP64 operations, no FMA, same reduction tree: bitwise
            assert np.array_equal(np.array(nrm), np.array(ref)), (nrm, ref)
            rref = rr.cpu().numpy()
            assert np.array_equal(r, rref)
            assert nrm[0] > 0 and nrm[1] > 0
    finally:
        L.gpu_finalize()


def test_noalloc_rejects_blocks_beyond_its_scratch(gpulib):
    import torch
    big = (C.c_int * 3)(2051, 2050, 3)  # 2049 * 2048 interior points > 4194304
    t = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = [C.c_double() for _ in range(4)]
    rc = L.lib().lester_norms_noalloc(big, *([L._p(t)] * 10), *[C.byref(o) for o in out], None)
    assert rc == -10
    msg = L.lib().lester_gpu_last_error().decode()
    assert "exceed" in msg and "4194304" in msg
