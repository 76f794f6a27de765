"""Summed-area table on the GPU (gme_sat / gme_sat_device / the reference's SOR)
against the oracle: ragged shapes around the strip width (256 columns) and the row
block (32 rows), row strides beyond n1 + 3, values that wrap, repeated calls, and a
size-independent check at 8192 x 8192 against the closed form."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (2, 3), (31, 31), (32, 33), (255, 1), (256, 32), (257, 64), (511, 95),
          (513, 97), (1000, 100), (3000, 70), (70, 3000), (5000, 300), (100000, 33)]


def _table(rng, n1, n2, ld, full_range=False):
    if full_range:
        return rng.integers(-2 ** 31, 2 ** 31, (n2 + 2, ld), dtype=np.int64).astype(np.int32)
    return rng.integers(0, 10000, (n2 + 2, ld)).astype(np.int32)


@pytest.mark.parametrize("n1,n2", SHAPES)
def test_sat_host_matches_oracle(gme_ctx, n1, n2):
    rng = np.random.default_rng(n1 * 7919 + n2)
    t = _table(rng, n1, n2, n1 + 3)
    want = O.sat(t, n1, n2)
    got = gme_ctx.sat(t.copy(), n1, n2)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("pad", [0, 1, 45])
def test_sat_device_strides_and_wrap(gme_ctx, pad):
    import torch
    rng = np.random.default_rng(100 + pad)
    n1, n2 = 777, 161
    ld = n1 + 1 + pad
    t = _table(rng, n1, n2, ld, full_range=True)
    want = O.sat(t, n1, n2)
    s = torch.cuda.Stream()  # an explicit stream: a null handle means the library's own
    with torch.cuda.stream(s):
        d = torch.from_numpy(t).cuda()
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        gme_ctx.sat_device(d.data_ptr(), n1, n2, ld, st.data_ptr(), s.cuda_stream)
        s.synchronize()
        assert int(st.item()) == 0
        np.testing.assert_array_equal(d.cpu().numpy(), want)


def test_sat_repeated_and_after_alignments(gme_ctx):
    """Carries are tagged per call: later calls (and plain alignments in between,
    which share the tagged scratch) never see an earlier call's words."""
    rng = np.random.default_rng(3)
    for i in range(4):
        n1, n2 = 600 + 37 * i, 90 + 11 * i
        t = _table(rng, n1, n2, n1 + 3)
        np.testing.assert_array_equal(gme_ctx.sat(t.copy(), n1, n2), O.sat(t, n1, n2))
        a = rng.integers(0, 4, 3000).astype(np.int32)
        b = rng.integers(0, 4, 2000).astype(np.int32)
        assert gme_ctx.align("ed", a, b).score == O.align(O.ED, a, b)["score"]


def test_sat_empty_is_noop(gme_ctx):
    t = np.arange(40, dtype=np.int32).reshape(5, 8)
    np.testing.assert_array_equal(gme_ctx.sat(t.copy(), 0, 3), t)
    np.testing.assert_array_equal(gme_ctx.sat(t.copy(), 4, 0), t)


def test_sat_reference_signature():
    """SOR(n1, n2, table, tX, tY) through its C form: the reference's layout of
    n2 + 2 rows of n1 + 3 ints; rows 1..n2 x columns 1..n1 get the table."""
    import gpumemefficient_gb300 as g
    L = g.lib()
    L.gme_ref_sor.restype = ctypes.c_int32
    L.gme_ref_sor.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]
    rng = np.random.default_rng(11)
    n1, n2 = 1024, 256
    t = _table(rng, n1, n2, n1 + 3)
    want = O.sat(t, n1, n2)
    got = t.copy()
    assert L.gme_ref_sor(n1, n2, got.ctypes.data) == 0
    np.testing.assert_array_equal(got, want)


def test_sat_8192_closed_form(gme_ctx):
    import torch
    rng = np.random.default_rng(8192)
    n1 = n2 = 8192
    t = _table(rng, n1, n2, n1 + 3)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        d = torch.from_numpy(t).cuda()
        gme_ctx.sat_device(d.data_ptr(), n1, n2, n1 + 3, 0, s.cuda_stream)
        s.synchronize()
        got = d.cpu().numpy()
    want = O.sat_py(t, n1, n2)
    np.testing.assert_array_equal(got, want)


def test_sat_tags_never_pass_for_band_rows():
    """SAT carries and the plain kernel's band rows share one tagged scratch buffer
    and one tag counter.  On one context whose scratch is already large (so nothing
    is regrown and no tag is reset): a big alignment, then SAT calls, each followed
    by an alignment with more bands than the tags the SAT calls took.  No SAT word
    may be read as a band row, so every score and last row equals the oracle's."""
    import os
    import gpumemefficient_gb300 as g
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(4242)
    with g.Context(0) as ctx:
        a = rng.integers(0, 4, 40000).astype(np.int32)
        b = rng.integers(0, 4, 40000).astype(np.int32)
        assert ctx.align("ed", a, b).score == O.align(O.ED, a, b, threads=threads)["score"]
        for i in range(3):
            n1, n2 = 2000 + 129 * i, 30000
            t = _table(rng, n1, n2, n1 + 3)
            np.testing.assert_array_equal(ctx.sat(t.copy(), n1, n2), O.sat(t, n1, n2))
            a = rng.integers(0, 4, 30000).astype(np.int32)
            b = rng.integers(0, 4, 60000).astype(np.int32)
            r = ctx.align("ed", a, b, last_row=True)
            o = O.align(O.ED, a, b, threads=threads)
            assert r.score == o["score"], i
            np.testing.assert_array_equal(r.last_row, o["last_row"])


TMA_SHAPES = [(1, 1, 4), (3, 5, 4), (127, 31, 128), (128, 32, 132), (129, 33, 132), (255, 64, 256),
              (256, 65, 260), (1000, 100, 1004), (4095, 97, 4096), (4096, 130, 4100), (70, 3000, 72),
              (5000, 300, 5004), (777, 161, 1024), (33, 64, 512)]


@pytest.mark.parametrize("n1,n2,ld", TMA_SHAPES)
def test_sat_tensor_map_path(gme_ctx, n1, n2, ld):
    """Rows of a multiple of 16 bytes take the tensor-map kernel (strips from column 0,
    boxes of 32 x 32 with 128-byte swizzle): ragged edges in both directions, padding
    columns and the extra rows past n2 come back as they were, values wrap."""
    import torch
    assert ld % 4 == 0
    rng = np.random.default_rng(n1 * 31 + n2 * 7 + ld)
    t = _table(rng, n1, n2, ld, full_range=True)
    want = O.sat(t, n1, n2)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        d = torch.from_numpy(t).cuda()
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        gme_ctx.sat_device(d.data_ptr(), n1, n2, ld, st.data_ptr(), s.cuda_stream)
        s.synchronize()
        assert int(st.item()) == 0
        got = d.cpu().numpy()
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got[:, n1 + 1:], t[:, n1 + 1:])  # padding columns untouched
    np.testing.assert_array_equal(got[n2 + 1:], t[n2 + 1:])        # rows past n2 untouched


def test_sat_unaligned_table_takes_the_copy_kernel(gme_ctx):
    """A table whose start is not 16-byte aligned (here 4 bytes in) runs on the cp.async
    kernel even with 16-byte rows, with the same result."""
    import torch
    rng = np.random.default_rng(77)
    n1, n2, ld = 600, 90, 604
    t = _table(rng, n1, n2, ld, full_range=True)
    want = O.sat(t, n1, n2)
    d = torch.zeros(t.size + 4, dtype=torch.int32, device="cuda")
    d[1:1 + t.size] = torch.from_numpy(t.reshape(-1)).cuda()
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    gme_ctx.sat_device(d.data_ptr() + 4, n1, n2, ld, st.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    np.testing.assert_array_equal(d[1:1 + t.size].cpu().numpy().reshape(t.shape), want)


def test_sat_tensor_map_large_closed_form(gme_ctx):
    """8192 x 8192 in a 16-byte-row layout (ld = n1 + 4) against the threaded oracle,
    twice, so that the tags of a second call meet the first call's words."""
    import torch
    rng = np.random.default_rng(5)
    n1 = n2 = 8192
    ld = n1 + 4
    t = rng.integers(0, 10000, (n2 + 2, ld)).astype(np.int32)
    want = O.sat_mt(t, n1, n2)
    for _ in range(2):
        d = torch.from_numpy(t).cuda()
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        gme_ctx.sat_device(d.data_ptr(), n1, n2, ld, st.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        np.testing.assert_array_equal(d.cpu().numpy(), want)
