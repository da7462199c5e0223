"""GPU parity of the engine against the oracle, through the C ABI (ctypes).

Tolerances (w = Omega / 4 pi):
  * build topology / skip links / leaf ranges / triangle order / centres / radii: bit-exact
    against the CPU restatement of the build (O3); FP64 moments within 1e-12 relative.
  * plain FP64 form vs O3 FP64 traversal of the same tree: |dw| <= 1e-10.
  * mixed form vs plain FP64 form (same tree, same beta): |dw| <= 1e-4 (the workload gate);
    observed values are far smaller and are asserted at <= 2e-6 on these inputs.
  * beta -> infinity (every triangle exact): FP64 form vs O1 brute force |dw| <= 1e-10,
    mixed vs O1 |dw| <= 1e-5.
  * is_inside agrees with the FP64 oracle on every point with |w - 0.5| > 1e-3.
"""
import ctypes as C
import math
import threading
from pathlib import Path

import numpy as np
import pytest

import lagrange_gb300 as fwn
from lagrange_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
FOUR_PI = 4 * math.pi
BOTH = fwn.RECORDS_F32 | fwn.RECORDS_F64


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    torch.cuda.set_device(0)
    return torch


def _q(eng, torch, Q, **kw):
    res = eng.query(torch.from_numpy(np.ascontiguousarray(Q, np.float32)).cuda(), **kw)
    torch.cuda.synchronize()
    return [r.cpu().numpy() if hasattr(r, "cpu") else r for r in res]


def _engine(V, F, **kw):
    kw.setdefault("records", BOTH | fwn.RECORDS_MOMENTS)
    return fwn.FastWindingNumber(V, F, **kw)


@pytest.mark.parametrize("leaf,builder", [(1, 0), (4, 0), (7, 0), (16, 0), (1, 1), (4, 1),
                                          (12, 1), (16, 1), (1, 2), (8, 2), (16, 2)])
def test_build_matches_cpu_restatement(torch_cuda, oracle_mod, leaf, builder):
    """Both builders (0: LBVH over Morton codes, 1: top-down longest-axis splits) against their
    CPU restatements: topology, skip links, leaf ranges, triangle order, centres and radii bit for
    bit; FP64 moments to 1e-12."""
    g = np.load(GOLDEN / "displaced.npz")
    eng = _engine(g["V"], g["F"], leaf_size=leaf, builder=builder)
    got = eng.export_tree()
    ref = oracle_mod.LbvhTree(g["V"], g["F"], leaf_size=leaf, builder=builder).export()
    for k in ("skip", "tri_begin", "tri_count", "sorted_tri", "mesh_root"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    np.testing.assert_array_equal(got["center_radius"], ref["center_radius"])
    m = eng.export_moments()
    scale = np.max(np.abs(ref["moments"]), axis=0) + 1e-300
    assert np.max(np.abs(m - ref["moments"]) / scale) <= 1e-12


def test_golden_uv_sphere(torch_cuda, oracle_mod):
    g = np.load(GOLDEN / "uv_sphere.npz")
    eng = _engine(g["V"], g["F"], leaf_size=4)  # the fixture was made with leaf 4
    w_mix, ins = _q(eng, torch_cuda, g["Q"])
    w32, _, w64 = _q(eng, torch_cuda, g["Q"], precision=fwn.PRECISION_FP64, omega_f64=True)
    np.testing.assert_allclose(w64, g["omega_lbvh_beta2"], rtol=0, atol=1e-10 * FOUR_PI)
    assert np.max(np.abs(w_mix - w64)) / FOUR_PI <= 2e-6
    we = g["omega_exact"] / FOUR_PI
    band = np.abs(we - 0.5) > 1e-3
    np.testing.assert_array_equal(ins[band].astype(bool), we[band] > 0.5)
    np.testing.assert_array_equal(ins[band], g["inside_ref"][band])
    # beta -> infinity: every triangle evaluated exactly
    _, _, x64 = _q(eng, torch_cuda, g["Q"], precision=fwn.PRECISION_FP64, omega_f64=True, beta=1e30)
    np.testing.assert_allclose(x64, g["omega_exact"], rtol=0, atol=1e-10 * FOUR_PI)
    xm, _ = _q(eng, torch_cuda, g["Q"], beta=1e30)
    assert np.max(np.abs(xm - g["omega_exact"])) / FOUR_PI <= 1e-5


@pytest.mark.parametrize("leaf,builder", [(1, 0), (4, 0), (16, 0), (4, 1), (12, 1)])
def test_displaced_near_surface(torch_cuda, oracle_mod, leaf, builder):
    g = np.load(GOLDEN / "displaced.npz")
    eng = _engine(g["V"], g["F"], leaf_size=leaf, builder=builder)
    ref = oracle_mod.LbvhTree(g["V"], g["F"], leaf_size=leaf, builder=builder).query_f64(
        g["Q"], beta=2.0)
    _, _, w64 = _q(eng, torch_cuda, g["Q"], precision=fwn.PRECISION_FP64, omega_f64=True)
    np.testing.assert_allclose(w64, ref, rtol=0, atol=1e-10 * FOUR_PI)
    for trav in (fwn.TRAVERSAL_THREAD, fwn.TRAVERSAL_WARP):
        wm, ins, st = _q(eng, torch_cuda, g["Q"], traversal=trav, stats=True)
        assert np.max(np.abs(wm - w64)) / FOUR_PI <= 2e-6
        assert st["tri_evals_fp64"] > 0      # near-surface queries use the FP64 near field
        assert st["far_evals"] > 0 and st["nodes_tested"] >= st["far_evals"]
    we = g["omega_exact"] / FOUR_PI
    band = np.abs(we - 0.5) > 1e-3
    _, ins = _q(eng, torch_cuda, g["Q"])
    np.testing.assert_array_equal(ins[band].astype(bool), we[band] > 0.5)


def test_golden_soup(torch_cuda, oracle_mod):
    """The defective soup (holes, flips, 1e-7-jittered duplicates; near-surface queries within
    1e-4): FP64 form vs the restated build's FP64 traversal, mixed vs FP64 form, beta -> infinity
    vs the brute force, and is_inside vs the FP64 form outside the band."""
    g = np.load(GOLDEN / "soup.npz")
    eng = _engine(g["V"], g["F"], leaf_size=8)
    w_mix, ins = _q(eng, torch_cuda, g["Q"])
    _, _, w64 = _q(eng, torch_cuda, g["Q"], precision=fwn.PRECISION_FP64, omega_f64=True)
    np.testing.assert_allclose(w64, g["omega_lbvh_beta2"], rtol=0, atol=1e-10 * FOUR_PI)
    assert np.max(np.abs(w_mix - w64)) / FOUR_PI <= 2e-6
    band = np.abs(w64 / FOUR_PI - 0.5) > 1e-3
    np.testing.assert_array_equal(ins[band].astype(bool), (w64 / FOUR_PI)[band] > 0.5)
    _, _, x64 = _q(eng, torch_cuda, g["Q"], precision=fwn.PRECISION_FP64, omega_f64=True, beta=1e30)
    np.testing.assert_allclose(x64, g["omega_exact"], rtol=0, atol=1e-10 * FOUR_PI)
    xm, _ = _q(eng, torch_cuda, g["Q"], beta=1e30)
    assert np.max(np.abs(xm - g["omega_exact"])) / FOUR_PI <= 1e-5


def test_schedules_and_sorting(torch_cuda):
    """Every schedule computes the same terms; only the Kahan summation order may differ (both
    schedules defer work in warp-dependent batches, so the Morton sort changes the order; the
    block size does not change warp composition, so it changes nothing)."""
    wl = W.displaced_icosphere_workload(nu=40, n_queries=20000)
    eng = _engine(wl.V, wl.F)
    a, ia = _q(eng, torch_cuda, wl.Q, traversal=fwn.TRAVERSAL_THREAD)
    b, ib = _q(eng, torch_cuda, wl.Q, traversal=fwn.TRAVERSAL_WARP)
    b2, _ = _q(eng, torch_cuda, wl.Q, traversal=fwn.TRAVERSAL_WARP, sort_queries=0)
    b3, _ = _q(eng, torch_cuda, wl.Q, traversal=fwn.TRAVERSAL_WARP)
    c, ic = _q(eng, torch_cuda, wl.Q, traversal=fwn.TRAVERSAL_THREAD, sort_queries=0)
    d, _ = _q(eng, torch_cuda, wl.Q, traversal=fwn.TRAVERSAL_THREAD, block_size=256)
    np.testing.assert_array_equal(b, b3)  # deterministic run to run
    np.testing.assert_array_equal(a, d)
    assert np.max(np.abs(b - b2)) / FOUR_PI <= 1e-6
    assert np.max(np.abs(a - b)) / FOUR_PI <= 1e-6
    assert np.max(np.abs(a - c)) / FOUR_PI <= 1e-6
    w = a / FOUR_PI
    band = np.abs(w - 0.5) > 1e-3
    np.testing.assert_array_equal(ia[band], ib[band])
    np.testing.assert_array_equal(ia[band], ic[band])
    # host (C-ABI copy-in/copy-out) path == device path with the same defaults
    dflt, idflt = _q(eng, torch_cuda, wl.Q)
    h, hi = eng.query(wl.Q)
    np.testing.assert_array_equal(h, dflt)
    np.testing.assert_array_equal(hi, idflt)


def test_edge_cases(torch_cuda, oracle_mod):
    # empty mesh: Omega = 0 everywhere
    e0 = fwn.FastWindingNumber(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32))
    w, ins = e0.query(np.array([[0, 0, 0], [1, 2, 3]], np.float32))
    assert np.all(w == 0) and np.all(ins == 0)
    # single triangle, query on a vertex / in its plane / above
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    F = np.array([[0, 1, 2]], np.int32)
    e1 = _engine(V, F)
    Q = np.array([[1, 0, 0], [2, 2, 0], [0.25, 0.25, 1], [0.25, 0.25, -1]], np.float32)
    w, _ = e1.query(Q)
    ref = oracle_mod.brute_f64(V, F, Q)
    assert np.all(np.isfinite(w))
    np.testing.assert_allclose(w, ref, atol=1e-6)
    # degenerate and duplicated triangles contribute as in the oracle
    Vd, Fd = W.uv_sphere(16, 8)
    Fd2 = np.concatenate([Fd, Fd[:5], [[0, 0, 1], [3, 3, 3]]]).astype(np.int32)
    e2 = _engine(Vd, Fd2)
    Q = np.random.default_rng(3).uniform(-1.5, 1.5, (2000, 3)).astype(np.float32)
    _, _, w64 = _q(e2, torch_cuda, Q, precision=fwn.PRECISION_FP64, omega_f64=True)
    np.testing.assert_allclose(w64, oracle_mod.LbvhTree(Vd, Fd2).query_f64(Q), atol=1e-9)
    # zero queries
    w, ins = e2.query(np.zeros((0, 3), np.float32))
    assert len(w) == 0 and len(ins) == 0
    # queries exactly on vertices: finite
    w, _ = e2.query(Vd[:50])
    assert np.all(np.isfinite(w))


def test_invalid_meshes(torch_cuda):
    V, F = W.uv_sphere(8, 4)
    Fb = F.copy()
    Fb[2, 2] = len(V)
    with pytest.raises(fwn.WindingError, match="out of range") as e:
        fwn.FastWindingNumber(V, Fb)
    assert e.value.status == 1
    Fn = F.copy()
    Fn[0, 0] = -1
    with pytest.raises(fwn.WindingError, match="out of range"):
        fwn.FastWindingNumber(V, Fn)
    Vn = V.copy()
    Vn[F[4, 1], 2] = np.inf
    with pytest.raises(fwn.WindingError, match="non-finite"):
        fwn.FastWindingNumber(Vn, F)
    # unreferenced NaN vertex is fine (not part of any triangle)
    Vx = np.concatenate([V, [[np.nan, 0, 0]]]).astype(np.float32)
    eng = fwn.FastWindingNumber(Vx, F)
    w, ins = eng.query(np.zeros((1, 3), np.float32))
    assert ins[0] == 1
    # FP64 form on an engine without FP64 records
    e32 = fwn.FastWindingNumber(V, F)
    with pytest.raises(fwn.WindingError, match="FP64 records"):
        e32.query(np.zeros((1, 3), np.float32), precision=fwn.PRECISION_FP64)


def test_query_order_presorted(torch_cuda):
    """fwn_query_order returns the query's own permutation: gathering the points in that order
    and querying with sort_queries=0 reproduces the sorted query bit for bit (both forms)."""
    torch = torch_cuda
    wl = W.displaced_icosphere_workload(nu=24, n_queries=50_000)
    eng = _engine(wl.V, wl.F)
    Q = torch.from_numpy(wl.Q).cuda()
    order = eng.query_order(Q)
    torch.cuda.synchronize()
    assert torch.equal(torch.sort(order).values, torch.arange(len(Q), device=order.device))
    Qs = Q[order]
    for prec in (fwn.PRECISION_MIXED, fwn.PRECISION_FP64):
        w, ins = eng.query(Q, precision=prec)
        ws, inss = eng.query(Qs, precision=prec, sort_queries=False)
        torch.cuda.synchronize()
        assert torch.equal(ws, w[order]) and torch.equal(inss, ins[order])
    # empty batch, forest handle refused
    assert eng.query_order(Q[:0]).numel() == 0
    fo = W.batched_forest_workload(n_meshes=2, seed=1, f_lo=100, f_hi=200, q_lo=5, q_hi=10)
    forest = fwn.Forest(fo.V, fo.voff, fo.F, fo.foff)
    buf = torch.empty(4, dtype=torch.int32, device=Q.device)
    with pytest.raises(fwn.WindingError, match="forest") as e:
        fwn._check(fwn.library().fwn_query_order(forest._h, C.c_void_p(Q.data_ptr()), 4,
                                                 C.c_void_p(buf.data_ptr()), None))
    assert e.value.status == 1


def test_host_query_large_batch(torch_cuda):
    """fwn_query_host on a 4.5M-point batch (pinned and pageable host buffers, one output or
    both) equals the device query bit for bit."""
    torch = torch_cuda
    V, F = W.icosphere(12)
    eng = _engine(V.astype(np.float32), F)
    Q = np.random.default_rng(8).uniform(-1.3, 1.3, (4_500_000, 3)).astype(np.float32)
    wd, idv = eng.query(torch.from_numpy(Q).cuda())
    torch.cuda.synchronize()
    wd, idv = wd.cpu().numpy(), idv.cpu().numpy()
    wh, ih = eng.query(Q)  # pageable numpy buffers
    np.testing.assert_array_equal(wh, wd)
    np.testing.assert_array_equal(ih, idv)
    Qp = torch.from_numpy(Q).pin_memory()
    wp = torch.empty(len(Q), dtype=torch.float32).pin_memory()
    ip = torch.empty(len(Q), dtype=torch.uint8).pin_memory()
    fwn._check(fwn.library().fwn_query_host(eng.handle, C.c_void_p(Qp.data_ptr()), len(Q),
                                            C.c_void_p(wp.data_ptr()), C.c_void_p(ip.data_ptr())))
    np.testing.assert_array_equal(wp.numpy(), wd)
    np.testing.assert_array_equal(ip.numpy(), idv)
    # one output only
    fwn._check(fwn.library().fwn_query_host(eng.handle, C.c_void_p(Qp.data_ptr()), len(Q), None,
                                            C.c_void_p(ip.data_ptr())))
    np.testing.assert_array_equal(ip.numpy(), idv)


def test_concurrent_queries_one_handle(torch_cuda):
    wl = W.displaced_icosphere_workload(nu=20, n_queries=5000)
    eng = _engine(wl.V, wl.F)
    ref, _ = eng.query(wl.Q)
    out = [None] * 8
    errs = []

    def run(i):
        try:
            out[i] = eng.query(wl.Q)[0]
        except Exception as ex:  # pragma: no cover
            errs.append(ex)

    ts = [threading.Thread(target=run, args=(i,)) for i in range(8)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errs
    for o in out:
        np.testing.assert_array_equal(o, ref)


@pytest.mark.parametrize("builder", [0, 1, 2])
def test_forest_matches_cpu_restatement(torch_cuda, oracle_mod, builder):
    fo = W.batched_forest_workload(n_meshes=9, seed=11, f_lo=100, f_hi=20000, q_lo=50, q_hi=3000)
    # add an empty mesh in the middle
    voff = np.insert(fo.voff, 4, fo.voff[4])
    foff = np.insert(fo.foff, 4, fo.foff[4])
    qoff = np.insert(fo.qoff, 4, fo.qoff[4])
    forest = fwn.Forest(fo.V, voff, fo.F, foff, records=BOTH, leaf_size=8, builder=builder)
    got = forest.export_tree()
    lb = oracle_mod.LbvhTree(fo.V, fo.F, leaf_size=8, voff=voff, foff=foff, builder=builder)
    ref = lb.export()
    for k in ("skip", "tri_begin", "tri_count", "sorted_tri", "mesh_root"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    np.testing.assert_array_equal(got["center_radius"], ref["center_radius"])
    import torch
    Qd = torch.from_numpy(fo.Q).cuda()
    w, ins = forest.query_forest(Qd, qoff)
    w64, _ = forest.query_forest(Qd, qoff, precision=fwn.PRECISION_FP64)
    torch.cuda.synchronize()
    w, w64, ins = w.cpu().numpy(), w64.cpu().numpy(), ins.cpu().numpy()
    qmesh = np.repeat(np.arange(len(qoff) - 1), np.diff(qoff)).astype(np.int32)
    r = lb.query_f64(fo.Q, beta=2.0, qmesh=qmesh)
    np.testing.assert_allclose(w64, r, rtol=0, atol=1e-6)  # float output of the FP64 form
    assert np.max(np.abs(w - w64)) / FOUR_PI <= 2e-6
    # closed meshes: inside flags match the FP64 oracle's
    wr = r / FOUR_PI
    band = np.abs(wr - 0.5) > 1e-3
    np.testing.assert_array_equal(ins[band].astype(bool), wr[band] > 0.5)


def test_forest_sort_key_widths(torch_cuda):
    """A forest query sorts on 32-bit keys (mesh id above a coarser level of the Hilbert index)
    while every mesh keeps at least 8 curve cells per query, else on 64-bit keys. 300 unit
    spheres (9 mesh bits, 23 Hilbert bits) with 1.1M queries on mesh 0 take the 64-bit path,
    with 2^20 the 32-bit one. Both match the FP64 form (per-mesh launches), and every query
    finds its own mesh: w is near 1 at its sphere's centre and near 0 outside it (the sanity
    bounds are loose, 1e-2; the parity bound is the FP64 comparison)."""
    torch = torch_cuda
    V0, F0 = W.icosphere(4)
    M = 300
    shifts = np.zeros((M, 3), np.float64)
    shifts[:, 0] = 3.0 * np.arange(M)
    V = np.concatenate([V0 + shifts[m] for m in range(M)]).astype(np.float32)
    F = np.tile(F0, (M, 1)).astype(np.int32)  # forest triangles index their own mesh's vertices
    voff = np.arange(M + 1, dtype=np.int64) * len(V0)
    foff = np.arange(M + 1, dtype=np.int64) * len(F0)
    forest = fwn.Forest(V, voff, F, foff, records=BOTH)
    rng = np.random.default_rng(12)
    for n_big in (1_100_000, 1 << 20):
        counts = np.full(M, 8)
        counts[0] = n_big
        qoff = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        Q = np.concatenate([rng.uniform(-1.4, 1.4, (c, 3)) + shifts[m]
                            for m, c in enumerate(counts)])
        Q[qoff[1:-1]] = shifts[1:]  # first query of every small mesh: its sphere's centre
        Q = Q.astype(np.float32)
        Qd = torch.from_numpy(Q).cuda()
        w, ins = forest.query_forest(Qd, qoff)
        w64, _ = forest.query_forest(Qd, qoff, precision=fwn.PRECISION_FP64)
        torch.cuda.synchronize()
        w, w64, ins = w.cpu().numpy(), w64.cpu().numpy(), ins.cpu().numpy()
        assert np.max(np.abs(w - w64)) / FOUR_PI <= 2e-6
        band = np.abs(w64 / FOUR_PI - 0.5) > 1e-3
        np.testing.assert_array_equal(ins[band].astype(bool), (w64 / FOUR_PI)[band] > 0.5)
        centres = qoff[1:-1]
        assert np.all(np.abs(w[centres] / FOUR_PI - 1.0) < 1e-2)
        r = np.linalg.norm(Q.astype(np.float64) - np.repeat(shifts, counts, axis=0), axis=1)
        outside = r > 1.2
        assert np.all(np.abs(w[outside]) / FOUR_PI < 1e-2)
        assert np.all(ins[r < 0.9] == 1) and np.all(ins[outside] == 0)


def test_graph_capture_replay(torch_cuda):
    """Queries captured in a CUDA graph (scratch becomes graph memory nodes) replay to the same
    bits as direct calls: one mesh through fwn_query, and a forest through fwn_forest_query with
    its query offsets in pinned host memory."""
    torch = torch_cuda
    L = fwn.library()
    wl = W.displaced_icosphere_workload(nu=30, n_queries=40_000)
    eng = _engine(wl.V, wl.F)
    Q = torch.from_numpy(wl.Q).cuda()
    ref_w, ref_i = eng.query(Q)
    fo = W.batched_forest_workload(n_meshes=6, seed=2, f_lo=500, f_hi=5000, q_lo=100, q_hi=4000)
    forest = fwn.Forest(fo.V, fo.voff, fo.F, fo.foff)
    Qf = torch.from_numpy(fo.Q).cuda()
    ref_fw, ref_fi = forest.query_forest(Qf, fo.qoff)
    torch.cuda.synchronize()
    w = torch.empty_like(ref_w)
    i = torch.empty_like(ref_i)
    fw = torch.empty_like(ref_fw)
    fi = torch.empty_like(ref_fi)
    qoff = torch.from_numpy(fo.qoff.astype(np.int64)).pin_memory()
    opts = fwn._opts(precision=fwn.PRECISION_MIXED)

    def calls(stream):
        sp = C.c_void_p(stream.cuda_stream)
        fwn._check(L.fwn_query(eng.handle, C.c_void_p(Q.data_ptr()), len(Q), C.c_void_p(w.data_ptr()),
                               C.c_void_p(i.data_ptr()), sp))
        fwn._check(L.fwn_forest_query(forest.handle, C.c_void_p(Qf.data_ptr()),
                                      C.c_void_p(qoff.data_ptr()), C.c_void_p(fw.data_ptr()),
                                      C.c_void_p(fi.data_ptr()), C.byref(opts), sp))

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        calls(side)  # warm-up outside the capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        calls(torch.cuda.current_stream())
    for _ in range(2):
        w.zero_()
        fw.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(w, ref_w) and torch.equal(i, ref_i)
        assert torch.equal(fw, ref_fw) and torch.equal(fi, ref_fi)


def test_query_order_is_a_hilbert_curve(torch_cuda):
    """The query sort key is a Hilbert index: points at the centres of an aligned 16^3 block of
    sort cells come out as a path whose consecutive cells are face neighbours (a Morton order
    would jump)."""
    torch = torch_cuda
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], np.float32)
    F = np.array([[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 4]], np.int32)  # bbox [0, 1]^3
    eng = fwn.FastWindingNumber(V, F)
    # the sort frame is the bbox grown by 25% per side, 1024 cells per axis
    cell = 1.5 / 1024
    idx = np.stack(np.meshgrid(*[np.arange(16)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pts = (-0.25 + (idx + 0.5) * cell).astype(np.float32)
    order = eng.query_order(torch.from_numpy(pts).cuda()).cpu().numpy()
    path = idx[order]
    steps = np.abs(np.diff(path, axis=0)).sum(1)
    assert np.all(steps == 1)


@pytest.mark.parametrize("scale,shift", [(2.0 ** -13, 0.0), (2.0 ** 13, 0.0), (1.0, 1e3),
                                         (2.0 ** -7, -50.0)])
def test_scale_and_translation(torch_cuda, scale, shift):
    """Winding numbers do not depend on the mesh's scale or position. After scaling and
    translating (coordinates rounded to float), the mixed form stays within the parity tolerance
    of the FP64 form (differences of nearby floats are exact, and the FP64 near-field radius
    scales with the bbox). Mapped back to the original units (exactly: power-of-two scales,
    exact float subtractions), the same geometry gives the same inside/outside answers."""
    torch = torch_cuda
    wl = W.displaced_icosphere_workload(nu=24, n_queries=30_000)
    V = (wl.V.astype(np.float64) * scale + shift).astype(np.float32)
    Q = (wl.Q.astype(np.float64) * scale + shift).astype(np.float32)
    eng = _engine(V, wl.F)
    w, ins = _q(eng, torch, Q)
    _, _, w64 = _q(eng, torch, Q, precision=fwn.PRECISION_FP64, omega_f64=True)
    assert np.max(np.abs(w - w64)) / FOUR_PI <= 2e-6
    band = np.abs(w64 / FOUR_PI - 0.5) > 1e-3
    np.testing.assert_array_equal(ins[band].astype(bool), (w64 / FOUR_PI)[band] > 0.5)
    Vb = (V.astype(np.float64) - shift) / scale
    Qb = (Q.astype(np.float64) - shift) / scale
    assert np.array_equal(Vb.astype(np.float32), Vb) and np.array_equal(Qb.astype(np.float32), Qb)
    base = _engine(Vb.astype(np.float32), wl.F)
    _, _, b64 = _q(base, torch, Qb.astype(np.float32), precision=fwn.PRECISION_FP64, omega_f64=True)
    # the two trees can differ (Morton cells of rounded centroids), so their far-field
    # truncation differs by up to ~5e-3 in w; the side of the surface does not
    clear = np.abs(b64 / FOUR_PI - 0.5) > 0.05
    np.testing.assert_array_equal(ins[clear].astype(bool), (b64 / FOUR_PI)[clear] > 0.5)


def test_non_finite_queries(torch_cuda):
    """NaN / inf query points do not disturb the other points of the batch or the call: a NaN
    point fails every far test, walks the whole tree and returns NaN (inside 0); the finite
    points return what they return alone, with either schedule."""
    torch = torch_cuda
    V, F = W.icosphere(8)
    eng = _engine(V.astype(np.float32), F)
    Q = np.random.default_rng(2).uniform(-1.5, 1.5, (256, 3)).astype(np.float32)
    bad = Q.copy()
    bad[::7, 0] = np.nan
    bad[3::11, 1] = np.inf
    bad[5::13, 2] = -np.inf
    nonfin = ~np.isfinite(bad).all(1)
    for trav in (fwn.TRAVERSAL_WARP, fwn.TRAVERSAL_THREAD):
        ref, iref = _q(eng, torch, Q, traversal=trav, sort_queries=0)
        w, ins = _q(eng, torch, bad, traversal=trav, sort_queries=0)
        if trav == fwn.TRAVERSAL_WARP:  # a lane's path and sum order ignore its neighbours
            np.testing.assert_array_equal(w[~nonfin], ref[~nonfin])
        else:  # the thread schedule batches leaves across lanes: only the sum order may move
            np.testing.assert_allclose(w[~nonfin], ref[~nonfin], rtol=0, atol=1e-5)
        clear = ~nonfin & (np.abs(ref / FOUR_PI - 0.5) > 1e-3)
        np.testing.assert_array_equal(ins[clear], iref[clear])
        assert np.all(ins[np.isnan(w)] == 0)
    w, ins = _q(eng, torch, bad)  # sorted: NaN keys fall in one cell, no error
    assert np.all(np.isfinite(w[~nonfin]))


def test_warp_schedule_variants_agree(torch_cuda):
    """Every warp-schedule variant (1-7: one or two queries per lane, register caps, paired
    f32x2 Taylor terms, structure-of-arrays records) computes the same terms in the same order
    with explicit roundings: the results equal variant 3's bit for bit (and the FP64 form's
    within 2e-6). The allocation-free entry point follows the handle's variant too."""
    torch = torch_cuda
    wl = W.displaced_icosphere_workload(nu=40, n_queries=50_000)
    Q = torch.from_numpy(wl.Q).cuda()
    ref = None
    for tuning in (3, 1, 2, 4, 5, 6, 7):
        eng = _engine(wl.V, wl.F, tuning=tuning)
        w, ins = _q(eng, torch, wl.Q)
        if ref is None:
            ref, iref = w, ins
            _, _, w64 = _q(eng, torch, wl.Q, precision=fwn.PRECISION_FP64, omega_f64=True)
            assert np.max(np.abs(w - w64)) / FOUR_PI <= 2e-6
        np.testing.assert_array_equal(w, ref, err_msg=f"variant {tuning}")
        np.testing.assert_array_equal(ins, iref, err_msg=f"variant {tuning}")
        if tuning == 4:
            L = fwn.library()
            wn = torch.empty_like(Q[:, 0])
            inn = torch.empty(len(Q), dtype=torch.uint8, device=Q.device)
            fwn._check(L.fwn_query_noalloc(eng.handle, C.c_void_p(Q.data_ptr()), len(Q),
                                           C.c_void_p(wn.data_ptr()), C.c_void_p(inn.data_ptr()),
                                           None))
            torch.cuda.synchronize()
            np.testing.assert_array_equal(wn.cpu().numpy(), w)


@pytest.mark.parametrize("leaf", [4, 12])
def test_fp64_warp_schedule_matches_thread_form(torch_cuda, oracle_mod, leaf):
    """The FP64 form on the warp cursor sums the same terms in the same order as the plain
    thread form: equal to it to 1e-12 in w and within 1e-10 of the FP64 restatement (O3), near
    the surface and in the box; at beta -> infinity within 1e-10 of the brute force (O1)."""
    g = np.load(GOLDEN / "displaced.npz")
    eng = _engine(g["V"], g["F"], leaf_size=leaf)
    Q = g["Q"]
    _, _, thr = _q(eng, torch_cuda, Q, precision=fwn.PRECISION_FP64,
                   traversal=fwn.TRAVERSAL_THREAD, omega_f64=True)
    w32, ins, wrp = _q(eng, torch_cuda, Q, precision=fwn.PRECISION_FP64,
                       traversal=fwn.TRAVERSAL_WARP, omega_f64=True)
    assert np.max(np.abs(wrp - thr)) / FOUR_PI <= 1e-12
    o3 = oracle_mod.LbvhTree(g["V"], g["F"], leaf_size=leaf).query_f64(Q, beta=2.0)
    assert np.max(np.abs(wrp - o3)) / FOUR_PI <= 1e-10
    np.testing.assert_array_equal(w32, wrp.astype(np.float32))
    np.testing.assert_array_equal(ins, (w32.astype(np.float64) > 2 * math.pi).astype(np.uint8))
    _, _, wx = _q(eng, torch_cuda, Q, precision=fwn.PRECISION_FP64, traversal=fwn.TRAVERSAL_WARP,
                  beta=1e30, omega_f64=True)
    assert np.max(np.abs(wx - g["omega_exact"])) / FOUR_PI <= 1e-10


def test_split_builder_degenerate_geometry(torch_cuda, oracle_mod):
    """The top-down builder on inputs that defeat midpoint splits: 300 copies of one triangle
    (every centroid equal), a flat grid (one axis of zero extent) and a cluster of nearly equal
    centroids (the midpoint rounds onto the low end) fall back to splits by position, and the
    device tree still equals its CPU restatement bit for bit."""
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    V1 = np.tile(tri, (300, 1))
    F1 = np.arange(900, dtype=np.int32).reshape(300, 3)
    g = np.stack(np.meshgrid(np.arange(20), np.arange(20), indexing="ij"), -1).reshape(-1, 2)
    V2 = np.concatenate([g, np.zeros((len(g), 1))], 1).astype(np.float32)
    q = np.arange(19)
    a = (q[:, None] * 20 + q[None, :]).ravel()
    F2 = np.concatenate([np.stack([a, a + 20, a + 1], 1), np.stack([a + 1, a + 20, a + 21], 1)]).astype(np.int32)
    eps = np.float32(1.0) + np.arange(40, dtype=np.float32) * np.finfo(np.float32).eps
    V3 = np.concatenate([np.stack([eps, eps, eps], 1),
                         np.stack([eps + 1, eps, eps], 1),
                         np.stack([eps, eps + 1, eps], 1)]).astype(np.float32)
    F3 = np.stack([np.arange(40), np.arange(40) + 40, np.arange(40) + 80], 1).astype(np.int32)
    for V, F in ((V1, F1), (V2, F2), (V3, F3)):
        for leaf in (1, 4):
            eng = _engine(V, F, leaf_size=leaf, builder=1)
            got = eng.export_tree()
            ref = oracle_mod.LbvhTree(V, F, leaf_size=leaf, builder=1).export()
            for k in ("skip", "tri_begin", "tri_count", "sorted_tri", "mesh_root"):
                np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
            np.testing.assert_array_equal(got["center_radius"], ref["center_radius"])
            assert got["tri_count"].max() <= leaf


@pytest.mark.parametrize("leaf,builder", [(1, 1), (8, 1), (16, 1), (1, 2), (8, 2)])
def test_split_builder_finisher_boundaries(torch_cuda, oracle_mod, leaf, builder):
    """The top-down builders hand every segment of at most 1024 triangles to a per-block
    finisher in shared memory. Meshes on either side of that size (1024 / 1025, 2048 / 2049
    triangles, scattered random triangles), a mesh of 1024 and one of 3000 copies of a single
    triangle (every split by position, inside the finisher and before it) and small meshes, in
    one forest and one at a time: the device trees equal their CPU restatement bit for bit."""
    rng = np.random.default_rng(5)
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    meshes = []
    for nf in (1024, 1025, 2048, 2049, 513, 9, 8, 1):
        V = rng.uniform(-1, 1, size=(3 * nf, 3)).astype(np.float32)
        meshes.append((V, np.arange(3 * nf, dtype=np.int32).reshape(nf, 3)))
    for nf in (1024, 3000):
        meshes.append((np.tile(tri, (nf, 1)), np.arange(3 * nf, dtype=np.int32).reshape(nf, 3)))
    voff = np.concatenate([[0], np.cumsum([len(v) for v, _ in meshes])]).astype(np.int64)
    foff = np.concatenate([[0], np.cumsum([len(f) for _, f in meshes])]).astype(np.int64)
    V = np.concatenate([v for v, _ in meshes])
    F = np.concatenate([f for _, f in meshes])
    keys = ("skip", "tri_begin", "tri_count", "sorted_tri", "mesh_root")
    forest = fwn.Forest(V, voff, F, foff, records=BOTH, leaf_size=leaf, builder=builder)
    got = forest.export_tree()
    ref = oracle_mod.LbvhTree(V, F, leaf_size=leaf, voff=voff, foff=foff, builder=builder).export()
    for k in keys:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    np.testing.assert_array_equal(got["center_radius"], ref["center_radius"])
    for Vm, Fm in meshes[:2] + meshes[-2:]:
        got = _engine(Vm, Fm, leaf_size=leaf, builder=builder).export_tree()
        ref = oracle_mod.LbvhTree(Vm, Fm, leaf_size=leaf, builder=builder).export()
        for k in keys:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
        np.testing.assert_array_equal(got["center_radius"], ref["center_radius"])
        assert got["tri_count"].max() <= leaf


@pytest.mark.parametrize("builder", [0, 1, 2])
def test_save_load_round_trip(torch_cuda, tmp_path, builder):
    """An engine written with fwn_save and read back with fwn_load has the same tree and answers
    every query with the same bits (mixed and FP64 forms); a forest with an empty mesh too. A
    file with one payload byte flipped is refused by its checksum."""
    g = np.load(GOLDEN / "displaced.npz")
    eng = _engine(g["V"], g["F"], leaf_size=8, builder=builder, records=BOTH)
    path = tmp_path / "eng.fwn"
    eng.save(path)
    back = fwn.FastWindingNumber.load(path)
    a, b = eng.export_tree(), back.export_tree()
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    for kw in ({}, {"precision": fwn.PRECISION_FP64, "omega_f64": True}):
        ra, rb = _q(eng, torch_cuda, g["Q"], **kw), _q(back, torch_cuda, g["Q"], **kw)
        for x, y in zip(ra, rb):
            np.testing.assert_array_equal(x, y)
    raw = bytearray(path.read_bytes())
    raw[len(raw) // 2] ^= 0x40
    bad = tmp_path / "bad.fwn"
    bad.write_bytes(bytes(raw))
    with pytest.raises(fwn.WindingError, match="corrupt"):
        fwn.FastWindingNumber.load(bad)
    fo = W.batched_forest_workload(n_meshes=5, seed=13, f_lo=200, f_hi=3000, q_lo=50, q_hi=500)
    voff = np.insert(fo.voff, 2, fo.voff[2])
    foff = np.insert(fo.foff, 2, fo.foff[2])
    qoff = np.insert(fo.qoff, 2, fo.qoff[2])
    forest = fwn.Forest(fo.V, voff, fo.F, foff, leaf_size=8, builder=builder)
    forest.save(tmp_path / "forest.fwn")
    f2 = fwn.Forest.load(tmp_path / "forest.fwn")
    Qd = torch_cuda.from_numpy(fo.Q).cuda()
    w1, i1 = forest.query_forest(Qd, qoff)
    w2, i2 = f2.query_forest(Qd, qoff)
    torch_cuda.cuda.synchronize()
    assert torch_cuda.equal(w1, w2) and torch_cuda.equal(i1, i2)


@pytest.mark.parametrize("builder", [0, 1, 2])
def test_fp32_records_round_fp64_records(torch_cuda, builder):
    """Every coefficient of an FP32 node record is its FP64 record's value rounded to nearest
    even (the build converts on the integer pipes; numpy's cast is the IEEE reference), and the
    centre and radius, float values by construction, are equal."""
    g = np.load(GOLDEN / "displaced.npz")
    eng = _engine(g["V"], g["F"], leaf_size=8, builder=builder, records=BOTH)
    n = eng.export_nodes()
    f32, f64 = n["f32"], n["f64"]
    pairs = [(slice(0, 4), slice(0, 4)),      # P, r
             (slice(7, 8), slice(6, 7)),      # trM1
             (slice(8, 14), slice(7, 13)),    # N, W
             (slice(14, 20), slice(13, 19)),  # C
             (slice(20, 30), slice(19, 29))]  # D
    for a, b in pairs:
        np.testing.assert_array_equal(f32[:, a], f64[:, b].astype(np.float32))
    np.testing.assert_array_equal(f32[:, 0:4].astype(np.float64), f64[:, 0:4])
    assert np.count_nonzero(f32[:, 8:30]) > 0.9 * f32[:, 8:30].size


def test_known_answers_on_the_engine(torch_cuda):
    """The closed-form cases on the GPU engine, mixed and FP64 forms: a closed sphere gives w = 1
    inside and 0 outside, reversed orientation gives -w, two disjoint spheres add, a sphere
    nested in another gives 2, the unit cube gives |w| = 1 at its centre and an open box 5/6
    (within the beta = 2 far-field error for the tree, 1e-9 with beta -> infinity)."""
    V, F = W.uv_sphere()
    Q = np.array([[0, 0, 0], [0.3, -0.2, 0.5], [2, 0, 0], [0, 0, -1.2]], np.float32)
    for kw, tol in (({}, 1e-2), ({"beta": 1e30}, 1e-6)):
        w, ins = _q(_engine(V, F), torch_cuda, Q, **kw)
        np.testing.assert_allclose(w / FOUR_PI, [1, 1, 0, 0], atol=tol)
        np.testing.assert_array_equal(ins, [1, 1, 0, 0])
        wr, insr = _q(_engine(V, F[:, [0, 2, 1]]), torch_cuda, Q, **kw)
        np.testing.assert_allclose(wr, -w, atol=tol * FOUR_PI)
        assert not insr.any()
    V2 = np.concatenate([V, V + np.float32(3.0), V * np.float32(0.5)])
    F2 = np.concatenate([F, F + len(V), F + 2 * len(V)]).astype(np.int32)
    Q2 = np.array([[0.1, 0, 0], [3, 3, 3], [1.5, 1.5, 1.5], [0.8, 0, 0]], np.float32)
    e2 = _engine(V2, F2)
    for kw, tol in (({}, 1e-2), ({"beta": 1e30}, 1e-6)):
        w, _ = _q(e2, torch_cuda, Q2, **kw)
        np.testing.assert_allclose(w / FOUR_PI, [2, 1, 0, 1], atol=tol)
        _, _, w64 = _q(e2, torch_cuda, Q2, precision=fwn.PRECISION_FP64, omega_f64=True, **kw)
        np.testing.assert_allclose(w64 / FOUR_PI, [2, 1, 0, 1], atol=tol)
    cv = np.array([[x, y, z] for x in (0, 1) for y in (0, 1) for z in (0, 1)], np.float32)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    cf = np.array([t for a, b, c, d in quads for t in ((a, b, c), (a, c, d))], np.int32)
    cen = np.array([[0.5, 0.5, 0.5]], np.float32)
    for faces, want in ((cf, 1.0), (cf[2:], 5 / 6)):
        w, _ = _q(_engine(cv, faces), torch_cuda, cen, beta=1e30)
        assert abs(abs(w[0]) / FOUR_PI - want) < 1e-6


@pytest.mark.parametrize("builder", [0, 1])
def test_forest_many_ragged_meshes(torch_cuda, oracle_mod, builder):
    """3,000 meshes of 0 to 24 triangles (every fifth one empty, some without queries), with
    0 to 9 queries each: one forest build and one persistent query against the FP64 brute
    force of each mesh (beta -> infinity: exact sums, so the mixed form is within 1e-5)."""
    rng = np.random.default_rng(21)
    Vs, Fs, Qs = [], [], []
    for m in range(3000):
        nf = 0 if m % 5 == 0 else int(rng.integers(1, 25))
        nv = 3 * nf
        Vs.append(rng.normal(size=(nv, 3)).astype(np.float32) + np.float32(m % 7))
        Fs.append(np.arange(nv, dtype=np.int32).reshape(-1, 3))
        Qs.append(rng.normal(size=(int(rng.integers(0, 10)), 3)).astype(np.float32) + np.float32(m % 7))
    voff = np.concatenate([[0], np.cumsum([len(v) for v in Vs])]).astype(np.int64)
    foff = np.concatenate([[0], np.cumsum([len(f) for f in Fs])]).astype(np.int64)
    qoff = np.concatenate([[0], np.cumsum([len(q) for q in Qs])]).astype(np.int64)
    V, F, Q = np.concatenate(Vs), np.concatenate(Fs), np.concatenate(Qs)
    forest = fwn.Forest(V, voff, F, foff, records=BOTH, leaf_size=4, builder=builder)
    torch = torch_cuda
    Qd = torch.from_numpy(Q).cuda()
    w, ins = forest.query_forest(Qd, qoff, beta=1e30)
    w64, _ = forest.query_forest(Qd, qoff, precision=fwn.PRECISION_FP64, beta=1e30)
    torch.cuda.synchronize()
    w, w64, ins = w.cpu().numpy(), w64.cpu().numpy(), ins.cpu().numpy()
    ref = np.concatenate([oracle_mod.brute_f64(Vs[m], Fs[m], Qs[m]) if len(Qs[m]) else
                          np.zeros(0) for m in range(3000)])
    # the FP64 form's Omega is returned as float: rounding of up to half an ulp of |Omega|,
    # which reaches ~3e-6 for the overlapping random triangles here (|Omega| up to ~40)
    np.testing.assert_allclose(w64, ref, rtol=2e-7, atol=1e-6)
    np.testing.assert_allclose(w, ref, rtol=2e-7, atol=1e-5 * FOUR_PI)
    empty = np.repeat(np.arange(3000) % 5 == 0, np.diff(qoff))
    assert np.all(w[empty] == 0) and not ins[empty].any()


def test_query_host_batches_equal_single_calls(torch_cuda):
    """fwn_query_host_batches (batch b copied in while batch b - 1 is queried, its results copied
    out during batch b + 1) returns for every batch exactly what fwn_query_host returns for it:
    batches of varying size including an empty one and a single point, from numpy arrays and
    from pinned tensors, and with one output left out."""
    torch = torch_cuda
    g = np.load(GOLDEN / "displaced.npz")
    eng = _engine(g["V"], g["F"], leaf_size=8, builder=1, records=fwn.RECORDS_F32)
    rng = np.random.default_rng(8)
    lo, hi = g["V"].min(0), g["V"].max(0)
    batches = [rng.uniform(lo - 0.2, hi + 0.2, size=(k, 3)).astype(np.float32)
               for k in (5000, 0, 1, 70000, 3, 20000)]
    ref = [eng.query(b) for b in batches]  # numpy points: one fwn_query_host call each
    as_np = lambda x: x.numpy() if hasattr(x, "numpy") else x  # noqa: E731
    for inp in (batches, [torch.from_numpy(b).pin_memory() for b in batches]):
        out = eng.query_host_batches(inp)
        assert len(out) == len(batches)
        for (w, i), (rw, ri) in zip(out, ref):
            np.testing.assert_array_equal(as_np(w), rw)
            np.testing.assert_array_equal(as_np(i), ri)
    for (w, i), (rw, _) in zip(eng.query_host_batches(batches, inside=False), ref):
        assert i is None
        np.testing.assert_array_equal(w, rw)
    assert eng.query_host_batches([]) == []
