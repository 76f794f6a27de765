"""gme_align_device_noalloc: the allocation-free entry point, through the C ABI.

Some callers of this library cannot call cudaMalloc (they run inside another
runtime's memory pool, or in a plugin that must not allocate on its hot path).
gme_align_device_noalloc serves them from a static device array; this test checks
that, on two calls in a row, it returns exactly what gme_align_device returns
(integer scores: the tolerance is zero).  Collected last so that a failure here
does not hide the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_LEN = 8192  # GME_NOALLOC_MAX_LEN in include/gme.h


def _noalloc_fn():
    import gpumemefficient_gb300 as g
    L = g.lib()
    f = L.gme_align_device_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                  ctypes.POINTER(g.Scoring), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _run_both(ctx, kind, a, b, sc):
    import torch
    import gpumemefficient_gb300 as g
    f = _noalloc_fn()
    dev = torch.device("cuda", 0)
    da = torch.from_numpy(np.ascontiguousarray(a, np.int32)).to(dev)
    db = torch.from_numpy(np.ascontiguousarray(b, np.int32)).to(dev)
    outs = []
    for use_noalloc in (True, False):
        d_out = torch.zeros(32, dtype=torch.uint8, device=dev)
        d_row = torch.full((len(a) + 1,), -7, dtype=torch.int32, device=dev)
        d_col = torch.full((len(b) + 1,), -7, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        if use_noalloc:
            st = f(kind, da.data_ptr(), len(a), db.data_ptr(), len(b), ctypes.byref(sc),
                   d_out.data_ptr(), d_row.data_ptr(), d_col.data_ptr(), None)
            assert st == 0, st
        else:
            ctx.align_device(kind, da.data_ptr(), len(a), db.data_ptr(), len(b), d_out.data_ptr(),
                             sc=sc, d_last_row=d_row.data_ptr(), d_last_col=d_col.data_ptr())
        torch.cuda.synchronize()
        res = g.Result.from_buffer_copy(bytes(d_out.cpu().numpy()))
        assert res.status == 0
        outs.append((res.score, res.sw_max, res.sw_max_y, res.sw_max_x,
                     d_row.cpu().numpy(), d_col.cpu().numpy()))
    return outs


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_noalloc_matches_align_device_twice(kind):
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(404 + kind)
    with g.Context(0) as ctx:
        # two calls in a row with different shapes: the shared array keeps the
        # previous call's contents, which must not leak into the next result
        for n1, n2, alpha in [(3000, 2500, 4), (MAX_LEN, 700, 20)]:
            a = rng.integers(0, alpha, n1)
            b = rng.integers(0, alpha, n2)
            sc = g.scoring(ed_boundary=int(rng.integers(0, 2)))
            (s1, m1, y1, x1, r1, c1), (s2, m2, y2, x2, r2, c2) = _run_both(ctx, kind, a, b, sc)
            assert (s1, m1, y1, x1) == (s2, m2, y2, x2)
            np.testing.assert_array_equal(r1, r2)
            np.testing.assert_array_equal(c1, c2)


def test_noalloc_rejects_oversize():
    import gpumemefficient_gb300 as g
    f = _noalloc_fn()
    sc = g.scoring()
    # rejected before any device work: the pointers are never touched
    assert f(0, 1, MAX_LEN + 1, 1, 10, ctypes.byref(sc), 1, None, None, None) == 1
    assert f(0, 1, 10, 1, MAX_LEN + 1, ctypes.byref(sc), 1, None, None, None) == 1
