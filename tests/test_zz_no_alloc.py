"""The allocation-free count entry point, for callers that may not allocate
GPU memory themselves (an application that owns the device heap, a real-time
loop, a sandboxed plugin): tc_count_noalloc_i32 takes device pointers and a
stream and keeps all its scratch in one fixed device array inside libtc.

Called through the C ABI and compared with the allocating entry point
(tc_count) on two calls in a row; sizes beyond its limit must be refused.
This file sorts last so that a run stopping at the first failure has run
every other test first."""
import ctypes as C

import numpy as np
import pytest

import families
import oracle
import trianglecount_gb300 as tc
from trianglecount_gb300 import generators as gen

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 18
MAX_NNZ = 1 << 21


def _device_csr(torch, rp, col):
    d_rp = torch.from_numpy(np.ascontiguousarray(rp, np.int32)).cuda()
    d_col = torch.from_numpy(np.ascontiguousarray(col, np.int32)).cuda()
    return d_rp, d_col


def test_noalloc_matches_tc_count_twice_in_a_row(ctx):
    torch = pytest.importorskip("torch")
    lib = tc.lib()
    cases = [gen.rmat(14), gen.road(200), families.complete(600)[:2], gen.chung_lu(100000, 12.0, seed=31)]
    for src, dst in cases:
        orp, ocl, want = oracle.pipeline(src, dst)
        assert len(orp) - 1 <= MAX_ROWS and len(ocl) <= MAX_NNZ
        assert ctx.count(ctx.upload(orp, ocl)) == want  # the allocating entry point agrees
        d_rp, d_col = _device_csr(torch, orp, ocl)
        stream = torch.cuda.current_stream()
        for _ in range(2):  # the shared scratch keeps the previous call's contents
            d_out = torch.full((1,), -1, dtype=torch.int64, device="cuda")
            st = lib.tc_count_noalloc_i32(C.c_void_p(d_rp.data_ptr()), C.c_void_p(d_col.data_ptr()), len(orp) - 1,
                                          len(ocl), len(orp) - 1, C.c_void_p(d_out.data_ptr()),
                                          C.c_void_p(stream.cuda_stream))
            assert st == 0, lib.tc_last_error()
            stream.synchronize()
            assert int(d_out.item()) == want


def test_noalloc_partial_roots_and_limits(ctx):
    torch = pytest.importorskip("torch")
    lib = tc.lib()
    src, dst = gen.rmat(12)
    orp, ocl, _ = oracle.pipeline(src, dst)
    d_rp, d_col = _device_csr(torch, orp, ocl)
    d_out = torch.zeros(1, dtype=torch.int64, device="cuda")
    nr = (len(orp) - 1) // 3
    st = lib.tc_count_noalloc_i32(C.c_void_p(d_rp.data_ptr()), C.c_void_p(d_col.data_ptr()), len(orp) - 1, len(ocl),
                                  nr, C.c_void_p(d_out.data_ptr()), None)
    assert st == 0
    torch.cuda.synchronize()
    assert int(d_out.item()) == ctx.count(ctx.upload(orp, ocl, n_roots=nr))
    st = lib.tc_count_noalloc_i32(C.c_void_p(d_rp.data_ptr()), C.c_void_p(d_col.data_ptr()), MAX_ROWS + 1, len(ocl),
                                  0, C.c_void_p(d_out.data_ptr()), None)
    assert st == -4 and b"at most" in lib.tc_last_error()


def test_noalloc_in_order_on_a_second_stream():
    """Two different graphs counted one after the other on a non-default
    stream: each call clears what it needs of the shared scratch in that
    stream's order, whatever ran before it."""
    torch = pytest.importorskip("torch")
    lib = tc.lib()
    s2 = torch.cuda.Stream()
    graphs = [oracle.pipeline(*gen.rmat(14)), oracle.pipeline(*gen.road(200))]
    bufs = []
    with torch.cuda.stream(s2):
        for orp, ocl, _ in graphs:
            d_rp, d_col = _device_csr(torch, orp, ocl)
            bufs.append((d_rp, d_col, torch.full((1,), -1, dtype=torch.int64, device="cuda")))
    s2.synchronize()
    for (orp, ocl, _), (d_rp, d_col, d_out) in zip(graphs, bufs):
        st = lib.tc_count_noalloc_i32(C.c_void_p(d_rp.data_ptr()), C.c_void_p(d_col.data_ptr()), len(orp) - 1,
                                      len(ocl), len(orp) - 1, C.c_void_p(d_out.data_ptr()),
                                      C.c_void_p(s2.cuda_stream))
        assert st == 0, lib.tc_last_error()
    s2.synchronize()
    assert [int(b[2].item()) for b in bufs] == [want for _, _, want in graphs]
