"""Pins the CPU oracle (no GPU): closed-form solid angles, known winding numbers, the order-2
expansion's convergence rate, the committed golden vectors, and the invariants of the restated
LBVH. The reference's own tests pin no values (modules/winding/tests/
test_fast_winding_number.cpp:80-125), so these known-answer tests are what the oracle rests on.
"""
import math
from pathlib import Path

import numpy as np
import pytest

from lagrange_gb300 import workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden"
FOUR_PI = 4 * math.pi


def test_analytic_triangles(oracle_mod):
    g = np.load(GOLDEN / "analytic.npz")
    T, Q, O = g["tris"], g["queries"], g["omega"]
    got = np.array([oracle_mod.tri_solid_angle(t[0], t[1], t[2], q) for t, q in zip(T, Q)])
    i = 0
    while i < len(O):
        if i + 1 < len(O) and np.isnan(O[i + 1]):
            assert got[i] + got[i + 1] == pytest.approx(O[i], abs=1e-13)
            i += 2
        else:
            assert np.isfinite(got[i])
            assert got[i] == pytest.approx(O[i], abs=1e-13)
            i += 1


def test_golden_triangles_regression(oracle_mod):
    g = np.load(GOLDEN / "triangles.npz")
    got = [oracle_mod.tri_solid_angle(t[0], t[1], t[2], q) for t, q in zip(g["tris"], g["queries"])]
    np.testing.assert_allclose(got, g["omega"], rtol=0, atol=1e-14)


def test_closed_meshes_known_winding(oracle_mod):
    V, F = W.uv_sphere()
    Q = np.array([[0, 0, 0], [0.3, -0.2, 0.5], [2, 0, 0], [0, 0, -1.2]], np.float32)
    w = oracle_mod.brute_f64(V, F, Q) / FOUR_PI
    np.testing.assert_allclose(w, [1, 1, 0, 0], atol=1e-12)
    # reversed orientation gives -w
    w_rev = oracle_mod.brute_f64(V, F[:, [0, 2, 1]], Q) / FOUR_PI
    np.testing.assert_allclose(w_rev, -w, atol=1e-12)
    # two disjoint spheres: additive
    V2 = np.concatenate([V, V + np.float32(3.0)])
    F2 = np.concatenate([F, F + len(V)])
    Q2 = np.array([[0, 0, 0], [3, 3, 3], [1.5, 1.5, 1.5]], np.float32)
    np.testing.assert_allclose(oracle_mod.brute_f64(V2, F2, Q2) / FOUR_PI, [1, 1, 0], atol=1e-12)
    # unit cube from its centre, and an open box (one face removed) gives 5/6
    cv = np.array([[x, y, z] for x in (0, 1) for y in (0, 1) for z in (0, 1)], np.float32)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    cf = np.array([t for a, b, c, d in quads for t in ((a, b, c), (a, c, d))], np.int32)
    cen = np.array([[0.5, 0.5, 0.5]], np.float32)
    w_cube = oracle_mod.brute_f64(cv, cf, cen)[0] / FOUR_PI
    assert abs(abs(w_cube) - 1.0) < 1e-12
    w_open = oracle_mod.brute_f64(cv, cf[2:], cen)[0] / FOUR_PI
    assert abs(abs(w_open) - 5 / 6) < 1e-12


def test_golden_uv_sphere_regression(oracle_mod):
    g = np.load(GOLDEN / "uv_sphere.npz")
    wl = W.uv_sphere_workload(4096)
    np.testing.assert_array_equal(g["V"], wl.V)      # generator is bit-stable
    np.testing.assert_array_equal(g["F"], wl.F)
    np.testing.assert_array_equal(g["Q"], wl.Q)
    o1 = oracle_mod.brute_f64(g["V"], g["F"], g["Q"])
    np.testing.assert_allclose(o1, g["omega_exact"], rtol=0, atol=1e-12)
    o3 = oracle_mod.LbvhTree(g["V"], g["F"], leaf_size=4).query_f64(g["Q"], beta=2.0)
    np.testing.assert_allclose(o3, g["omega_lbvh_beta2"], rtol=0, atol=1e-12)
    # closed sphere: the exact winding number is 0 or 1 off the surface
    w = o1 / FOUR_PI
    r = np.linalg.norm(g["Q"].astype(np.float64), axis=1)
    off = np.abs(r - 1) > 0.05
    np.testing.assert_allclose(w[off], (r[off] < 1).astype(float), atol=1e-9)


def test_golden_soup_regression(oracle_mod):
    """The defective soup (holes, flipped and jittered duplicate faces): the generator is
    bit-stable and O1 / O3 reproduce the committed values; O3 at beta=2 stays within the
    truncation bound of O1, and the holes make the exact winding numbers fractional."""
    g = np.load(GOLDEN / "soup.npz")
    sp = W.defective_soup_workload(nu=20, n_queries=2048)
    for k in ("V", "F", "Q"):
        np.testing.assert_array_equal(g[k], getattr(sp, k))
    o1 = oracle_mod.brute_f64(g["V"], g["F"], g["Q"])
    np.testing.assert_allclose(o1, g["omega_exact"], rtol=0, atol=1e-12)
    o3 = oracle_mod.LbvhTree(g["V"], g["F"], leaf_size=8).query_f64(g["Q"], beta=2.0)
    np.testing.assert_allclose(o3, g["omega_lbvh_beta2"], rtol=0, atol=1e-12)
    assert np.max(np.abs(o3 - o1)) / FOUR_PI < 2e-2
    w = o1 / FOUR_PI
    assert np.sum((w > 0.05) & (w < 0.95)) > 10  # fractional winding numbers exist


def test_restated_reference_tree_accuracy(oracle_mod):
    """O2 (float Barill tree, beta=2) against the FP64 brute force, and its is_inside."""
    g = np.load(GOLDEN / "uv_sphere.npz")
    om, ins = oracle_mod.RefTree(g["V"], g["F"], 4).query(g["Q"], beta=2.0)
    w_exact = g["omega_exact"] / FOUR_PI
    assert np.max(np.abs(om / FOUR_PI - w_exact)) < 2e-2
    band = np.abs(w_exact - 0.5) > 1e-3
    assert np.array_equal(ins[band].astype(bool), w_exact[band] > 0.5)
    np.testing.assert_array_equal(ins, g["inside_ref"])


def test_lbvh_exact_equals_brute(oracle_mod):
    g = np.load(GOLDEN / "displaced.npz")
    lb = oracle_mod.LbvhTree(g["V"], g["F"], leaf_size=4)
    ex = lb.query_f64(g["Q"], exact=True)
    np.testing.assert_allclose(ex, g["omega_exact"], rtol=0, atol=1e-10)
    b2 = lb.query_f64(g["Q"], beta=2.0)
    assert np.max(np.abs(b2 - g["omega_exact"])) / FOUR_PI < 2e-2


def test_taylor_order2_convergence(oracle_mod):
    """Absolute far-field error of an order-2 expansion falls like D^-5 (x32 per doubling)."""
    P, F = W.icosphere(8)
    V = P.astype(np.float32)
    cen = P[F].mean(1)
    sel = np.argsort(np.linalg.norm(cen - cen[0], axis=1))[:16]
    Fp = F[sel]
    lb = oracle_mod.LbvhTree(V, Fp, leaf_size=16)
    assert lb.num_nodes == 1
    ex = lb.export()
    Pn, r = ex["center_radius"][0, :3], ex["center_radius"][0, 3]
    dirs = np.random.default_rng(0).normal(size=(64, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    errs = []
    for ratio in (4, 8, 16):
        Q = (Pn + dirs * ratio * r).astype(np.float32)
        errs.append(np.max(np.abs(lb.query_f64(Q, beta=1.0) - oracle_mod.brute_f64(V, Fp, Q))))
    assert errs[0] / errs[1] > 24 and errs[1] / errs[2] > 24


@pytest.mark.parametrize("leaf", [1, 3, 4, 16])
def test_lbvh_invariants(oracle_mod, leaf):
    g = np.load(GOLDEN / "displaced.npz")
    lb = oracle_mod.LbvhTree(g["V"], g["F"], leaf_size=leaf)
    ex = lb.export()
    E = lb.num_nodes
    skip, tb, tc = ex["skip"], ex["tri_begin"], ex["tri_count"]
    nf = len(g["F"])
    assert np.all(skip > np.arange(E)) and skip[0] == E
    assert np.all(skip <= E)
    # leaves cover every sorted slot exactly once, in DFS (= Morton) order
    leaves = np.nonzero(tc > 0)[0]
    assert np.all(tc[leaves] <= leaf)
    cover = np.concatenate([np.arange(tb[i], tb[i] + tc[i]) for i in leaves])
    np.testing.assert_array_equal(cover, np.arange(nf))
    assert sorted(ex["sorted_tri"].tolist()) == list(range(nf))
    # internal nodes: first child at i+1; subtree sizes consistent
    internal = np.nonzero(tc == 0)[0]
    assert np.all(skip[internal] > internal + 1)
    # radius bounds every vertex of the node's triangles
    V = g["V"].astype(np.float64)
    Fs = g["F"][ex["sorted_tri"]]
    for i in leaves[:200]:
        pts = V[Fs[tb[i]:tb[i] + tc[i]].reshape(-1)]
        d = np.linalg.norm(pts - ex["center_radius"][i, :3], axis=1)
        assert np.all(d <= ex["center_radius"][i, 3])
    # centres and radii are float values
    cr = ex["center_radius"]
    np.testing.assert_array_equal(cr, cr.astype(np.float32).astype(np.float64))


def test_lbvh_forest_matches_single(oracle_mod):
    """Each mesh of a forest is one subtree; a one-mesh forest equals the single build."""
    a = W.uv_sphere(16, 8)
    b = W.displaced_icosphere(6, 7)
    V = np.concatenate([a[0], b[0]])
    F = np.concatenate([a[1], b[1]])
    voff = [0, len(a[0]), len(V)]
    foff = [0, len(a[1]), len(F)]
    lb = oracle_mod.LbvhTree(V, F, leaf_size=4, voff=voff, foff=foff)
    ex = lb.export()
    roots = ex["mesh_root"]
    assert roots[0, 1] <= roots[1, 0] or roots[1, 1] <= roots[0, 0]
    Q = np.array([[0, 0, 0], [0.5, 0, 0], [3, 3, 3]], np.float32)
    w = lb.query_f64(Q, beta=2.0, qmesh=np.array([0, 0, 0])) / FOUR_PI
    np.testing.assert_allclose(w, [1, 1, 0], atol=2e-2)
    w1 = lb.query_f64(Q, beta=2.0, qmesh=np.array([1, 1, 1])) / FOUR_PI
    np.testing.assert_allclose(w1, [1, 1, 0], atol=2e-2)


def test_lbvh_rejects_bad_input(oracle_mod):
    V, F = W.uv_sphere(8, 4)
    Fb = F.copy()
    Fb[3, 1] = len(V)
    with pytest.raises(ValueError):
        oracle_mod.LbvhTree(V, Fb)
    Vb = V.copy()
    Vb[F[0, 0], 1] = np.nan
    with pytest.raises(ValueError):
        oracle_mod.LbvhTree(Vb, F)


@pytest.mark.parametrize("builder", [0, 1])
def test_tree_builders_structure_and_exact_limit(oracle_mod, builder):
    """Both restated builds give a DFS tree whose leaves hold every triangle once in <= leaf_size
    runs, with consistent skip links, and whose beta -> infinity traversal is the brute force."""
    d = W.displaced_icosphere_workload(nu=10, n_queries=300)
    for leaf in (1, 5, 12):
        t = oracle_mod.LbvhTree(d.V, d.F, leaf_size=leaf, builder=builder)
        ex = t.export()
        E = t.num_nodes
        skip, tb, tc = ex["skip"], ex["tri_begin"], ex["tri_count"]
        assert np.all(skip > np.arange(E)) and np.all(skip <= E)
        leaves = tc > 0
        assert tc.max() <= leaf and tc[leaves].sum() == len(d.F)
        covered = np.concatenate([np.arange(b, b + c) for b, c in zip(tb[leaves], tc[leaves])])
        np.testing.assert_array_equal(np.sort(covered), np.arange(len(d.F)))
        assert sorted(ex["sorted_tri"]) == list(range(len(d.F)))
        r = ex["center_radius"][:, 3]
        assert np.all(r >= 0) and np.all(np.isfinite(r))
    exact = oracle_mod.brute_f64(d.V, d.F, d.Q)
    w = oracle_mod.LbvhTree(d.V, d.F, leaf_size=8, builder=builder).query_f64(d.Q, beta=1e30)
    np.testing.assert_allclose(w, exact, rtol=0, atol=1e-10 * 4 * np.pi)


def test_o2_speed_build_matches_checker(oracle_mod):
    """The -O3 build of O2 that the timed CPU legs use gives the checker build's answers up to
    float contraction."""
    g = np.load(GOLDEN / "uv_sphere.npz")
    a, ia = oracle_mod.RefTree(g["V"], g["F"], 8).query(g["Q"][:2000], nthreads=2)
    b, ib = oracle_mod.RefTree(g["V"], g["F"], 8, fast=True).query(g["Q"][:2000], nthreads=2)
    assert np.max(np.abs(a.astype(np.float64) - b)) / (4 * np.pi) <= 1e-5
    band = np.abs(a / (4 * np.pi) - 0.5) > 1e-3
    np.testing.assert_array_equal(ia[band], ib[band])


def test_reference_engine_when_present(oracle_mod):
    """When a built reference is present under baseline/_ref, its own FastWindingNumber (through
    oracle/ref_shim.cpp) answers like the FP64 brute force on a closed sphere: is_inside equal
    outside the +-1e-3 band, |dw| within the beta = 2 truncation. Skipped otherwise, with why."""
    ok, why = oracle_mod.reference_available()
    if not ok:
        pytest.skip(why)
    g = np.load(GOLDEN / "uv_sphere.npz")
    om, ins = oracle_mod.ReferenceEngine(g["V"], g["F"]).query(g["Q"])
    exact = g["omega_exact"] / (4 * np.pi)
    assert np.max(np.abs(om / (4 * np.pi) - exact)) <= 1e-2
    band = np.abs(exact - 0.5) > 1e-3
    np.testing.assert_array_equal(ins[band].astype(bool), exact[band] > 0.5)


@pytest.mark.parametrize("leaf", [1, 8])
def test_split_builders_tree_invariants(oracle_mod, leaf):
    """The restated top-down builds (1: midpoints; 2: least-cost binned planes above 1024
    triangles): every triangle in exactly one leaf, leaves of at most leaf_size triangles,
    pre-order skip links (a node's subtree is the run of positions up to its skip), each internal
    node's range the union of its children's, and the binned rule changing the tree of a mesh
    large enough to use it."""
    wl = W.displaced_icosphere_workload(nu=40, n_queries=400)  # 32,000 triangles
    trees = {}
    for builder in (1, 2):
        ex = oracle_mod.LbvhTree(wl.V, wl.F, leaf_size=leaf, builder=builder).export()
        skip, tb, tc = ex["skip"], ex["tri_begin"], ex["tri_count"]
        E = len(skip)
        assert np.array_equal(np.sort(ex["sorted_tri"]), np.arange(len(wl.F)))
        leaves = tc > 0
        assert tc.max() <= leaf and tc[leaves].sum() == len(wl.F)
        # leaves tile the slots in order
        starts = tb[leaves]
        assert np.array_equal(starts, np.concatenate([[0], np.cumsum(tc[leaves])[:-1]]))
        assert np.all(skip[:-1] > np.arange(E - 1)) and skip[0] == E
        internal = np.flatnonzero(~leaves)
        assert np.all(skip[internal + 1] < skip[internal])  # the left child ends before its parent
        right = skip[internal + 1]
        assert np.all(skip[right] == skip[internal])          # the right child ends with it
        trees[builder] = ex
    assert not np.array_equal(trees[1]["sorted_tri"], trees[2]["sorted_tri"])
