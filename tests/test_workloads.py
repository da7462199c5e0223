"""Synthetic workload generators: sizes of the five workloads, closedness and orientation."""
import numpy as np

from lagrange_gb300 import workloads as W


def _edges_manifold_closed(F):
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    fwd = {tuple(x) for x in e.tolist()}
    # every directed edge has its opposite: closed and consistently oriented
    return all((b, a) in fwd for a, b in fwd) and len(fwd) == len(e)


def test_uv_sphere_sizes():
    V, F = W.uv_sphere(64, 32)
    assert V.shape == (1986, 3) and F.shape == (3968, 3)
    assert V.dtype == np.float32 and F.dtype == np.int32
    assert _edges_manifold_closed(F)
    wl = W.uv_sphere_workload()
    assert wl.Q.shape == (100_000, 3)
    assert wl.Q.min() >= -1.5 and wl.Q.max() <= 1.5


def test_icosphere_sizes_and_closed():
    for nu in (1, 2, 5, 9):
        P, F = W.icosphere(nu)
        assert P.shape == (10 * nu * nu + 2, 3)
        assert F.shape == (20 * nu * nu, 3)
        assert _edges_manifold_closed(F)
        a, b, c = P[F[:, 0]], P[F[:, 1]], P[F[:, 2]]
        assert np.all(np.sum(np.cross(b - a, c - a) * (a + b + c), 1) > 0)  # outward
    # the large workloads' triangle counts
    assert 20 * 316 ** 2 == 1_997_120 and 20 * 224 ** 2 == 1_003_520 and 20 * 500 ** 2 == 5_000_000


def test_torus_closed_outward():
    V, F, n, c = W.torus_grid(20, 8, 1.0, 0.3)
    assert F.shape == (2 * 20 * 8, 3)
    assert _edges_manifold_closed(F)
    a, b, cc = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    cen = (a + b + cc) / 3
    ring = cen.copy()
    ring[:, 2] = 0
    ring /= np.linalg.norm(ring, axis=1, keepdims=True)
    assert np.all(np.sum(np.cross(b - a, cc - a) * (cen - ring), 1) > 0)


def test_displaced_workload_small():
    wl = W.displaced_icosphere_workload(nu=12, n_queries=1000)
    assert wl.F.shape == (20 * 144, 3) and wl.Q.shape == (1000, 3)
    assert wl.near_mask.sum() == 500
    r = np.linalg.norm(wl.V.astype(np.float64), axis=1)
    assert 0.8 < r.min() and r.max() < 1.2
    wl2 = W.displaced_icosphere_workload(nu=12, n_queries=1000)
    np.testing.assert_array_equal(wl.Q, wl2.Q)


def test_defective_soup_small():
    wl = W.defective_soup_workload(nu=20, n_queries=2000)
    nf0 = 20 * 400
    kept = nf0 - nf0 // 10
    assert len(wl.F) == kept + kept // 200
    assert wl.F.max() < len(wl.V)


def test_forest_small():
    fo = W.batched_forest_workload(n_meshes=6, f_lo=200, f_hi=2000, q_lo=10, q_hi=100)
    assert len(fo.voff) == 7 and fo.foff[-1] == len(fo.F) and fo.qoff[-1] == len(fo.Q)
    for m in range(6):
        Fm = fo.F[fo.foff[m]:fo.foff[m + 1]]
        assert Fm.min() >= 0 and Fm.max() < fo.voff[m + 1] - fo.voff[m]


def test_voxel_grid():
    V, _ = W.uv_sphere(8, 4)
    G = W.voxel_grid(V, res=8)
    assert G.shape == (512, 3)
    assert np.all(np.diff(G[:8, 0]) > 0)  # x fastest
