"""fwn_query_noalloc: the query entry point that allocates no device memory.

It exists for callers that must not allocate GPU memory while they query (for instance a
voxelizer or renderer running under a fixed per-frame device budget, or code where a
cudaMalloc/cudaFree could fail or would stall other streams). Its sort buffers live in one fixed
region built into the library, which caps a call at FWN_NOALLOC_MAX_POINTS points.

These tests call it through the C ABI and compare it with fwn_query (same handle, same defaults)
on two calls in a row, so the second call runs on a region that still holds the first call's
contents. Tolerance as in the other parity tests: |dw| <= 1e-6 (w = Omega / 4 pi), identical
is_inside outside the +-1e-3 band. This file is collected last on purpose.
"""
import ctypes as C
import math
import re
from pathlib import Path

import numpy as np
import pytest

import lagrange_gb300 as fwn
from lagrange_gb300 import workloads as W

pytestmark = pytest.mark.gpu
FOUR_PI = 4 * math.pi
HEADER = Path(__file__).resolve().parent.parent / "include" / "fwn_gb300.h"


def max_points() -> int:
    m = re.search(r"#define FWN_NOALLOC_MAX_POINTS \(1 << (\d+)\)", HEADER.read_text())
    assert m, "FWN_NOALLOC_MAX_POINTS not found in the header"
    return 1 << int(m.group(1))


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _run(L, eng, Q, stream, noalloc: bool):
    import torch
    n = Q.shape[0]
    w = torch.full((n,), float("nan"), dtype=torch.float32, device=Q.device)
    ins = torch.full((n,), 7, dtype=torch.uint8, device=Q.device)
    if noalloc:
        st = L.fwn_query_noalloc(eng.handle, _ptr(Q), n, _ptr(w), _ptr(ins), stream)
    else:
        st = L.fwn_query(eng.handle, _ptr(Q), n, _ptr(w), _ptr(ins), stream)
    fwn._check(st)
    torch.cuda.synchronize()
    return w.cpu().numpy(), ins.cpu().numpy()


def _compare(w, ins, w_ref, ins_ref):
    assert np.all(np.isfinite(w))
    assert np.max(np.abs(w.astype(np.float64) - w_ref)) / FOUR_PI <= 1e-6
    band = np.abs(w_ref / FOUR_PI - 0.5) > 1e-3
    np.testing.assert_array_equal(ins[band], ins_ref[band])
    assert set(np.unique(ins)) <= {0, 1}


def test_noalloc_matches_fwn_query_two_calls_in_a_row():
    import torch
    torch.cuda.set_device(0)
    L = fwn.library()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    wl = W.displaced_icosphere_workload(nu=48, n_queries=300_000)
    eng = fwn.FastWindingNumber(wl.V, wl.F)
    Q = torch.from_numpy(wl.Q).cuda()
    w_ref, ins_ref = _run(L, eng, Q, stream, noalloc=False)
    for _ in range(2):
        w, ins = _run(L, eng, Q, stream, noalloc=True)
        _compare(w, ins, w_ref.astype(np.float64), ins_ref)
    # a different, smaller batch right after: the region still holds the larger batch's data
    Q2 = Q[7:1007].contiguous()
    w2_ref, i2_ref = _run(L, eng, Q2, stream, noalloc=False)
    for _ in range(2):
        w2, i2 = _run(L, eng, Q2, stream, noalloc=True)
        _compare(w2, i2, w2_ref.astype(np.float64), i2_ref)


def test_noalloc_at_the_size_limit_and_beyond():
    import torch
    torch.cuda.set_device(0)
    L = fwn.library()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    cap = max_points()
    wl = W.displaced_icosphere_workload(nu=24, n_queries=cap)
    eng = fwn.FastWindingNumber(wl.V, wl.F)
    Q = torch.from_numpy(wl.Q).cuda()
    assert Q.shape[0] == cap
    w_ref, ins_ref = _run(L, eng, Q, stream, noalloc=False)
    for _ in range(2):
        w, ins = _run(L, eng, Q, stream, noalloc=True)
        _compare(w, ins, w_ref.astype(np.float64), ins_ref)
    # one point over the limit is refused with a clear message, before any device work
    Qbig = torch.zeros((cap + 1, 3), dtype=torch.float32, device="cuda")
    out = torch.zeros(cap + 1, dtype=torch.float32, device="cuda")
    st = L.fwn_query_noalloc(eng.handle, _ptr(Qbig), cap + 1, _ptr(out), None, stream)
    assert st == 1
    buf = C.create_string_buffer(512)
    L.fwn_last_error(buf, 512)
    assert "FWN_NOALLOC_MAX_POINTS" in buf.value.decode()
    # no handle: NOT_BUILT
    assert L.fwn_query_noalloc(None, _ptr(Qbig), 1, _ptr(out), None, stream) == 6


def test_noalloc_allocates_nothing():
    """A warm fwn_query_noalloc call takes no memory from anywhere: the device's free memory
    (cudaMemGetInfo) and the library's scratch pool (reserved bytes, and the high-water mark of
    handed-out bytes, restarted just before) are unchanged across two calls. fwn_query, which
    does take stream-ordered scratch, moves the high-water mark: the check can see an allocation."""
    import torch
    torch.cuda.set_device(0)
    L = fwn.library()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    wl = W.displaced_icosphere_workload(nu=32, n_queries=200_000)
    eng = fwn.FastWindingNumber(wl.V, wl.F)
    Q = torch.from_numpy(wl.Q).cuda()
    n = Q.shape[0]
    w = torch.empty(n, dtype=torch.float32, device="cuda")
    ins = torch.empty(n, dtype=torch.uint8, device="cuda")
    fwn._check(L.fwn_query(eng.handle, _ptr(Q), n, _ptr(w), _ptr(ins), stream))  # pool exists
    fwn._check(L.fwn_query_noalloc(eng.handle, _ptr(Q), n, _ptr(w), _ptr(ins), stream))  # warm
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    p0 = fwn.scratch_pool_stats(0, reset_high=True)
    assert p0["reserved"] > 0 and p0["used_high"] == p0["used"]
    for _ in range(2):
        fwn._check(L.fwn_query_noalloc(eng.handle, _ptr(Q), n, _ptr(w), _ptr(ins), stream))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    p1 = fwn.scratch_pool_stats(0)
    assert free1 == free0
    assert p1["reserved"] == p0["reserved"]
    assert p1["used"] == p0["used"] and p1["used_high"] == p0["used"]
    # the same probe sees the ordinary query's scratch
    fwn._check(L.fwn_query(eng.handle, _ptr(Q), n, _ptr(w), _ptr(ins), stream))
    torch.cuda.synchronize()
    p2 = fwn.scratch_pool_stats(0)
    assert p2["used_high"] > p0["used"]
