"""Batched callers of the winding-number path:
* fwn_query_grid — the voxel sign pass of volume::mesh_to_volume
  (modules/volume/src/mesh_to_volume.cpp:156-183);
* fwn_orientation_criterion — modules/winding/examples/fix_orientation.cpp:75-115;
* sample_inside — modules/winding/examples/sample_points_in_mesh.cpp:59-76.
"""
import math

import numpy as np
import pytest

import lagrange_gb300 as fwn
from lagrange_gb300 import workloads as W

pytestmark = pytest.mark.gpu
FOUR_PI = 4 * math.pi


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    torch.cuda.set_device(0)
    return torch


@pytest.mark.parametrize("tuning", [0, 4])  # one voxel per lane (auto at this size), two per lane
def test_grid_equals_explicit_points(torch_cuda, tuning):
    torch = torch_cuda
    V, F = W.displaced_icosphere(40, 5)
    eng = fwn.FastWindingNumber(V, F, tuning=tuning)
    dims = (37, 29, 23)  # not multiples of the 4x4x2 or 4x4x4 brick
    lo, hi = V.min(0).astype(np.float64), V.max(0).astype(np.float64)
    c, h = (lo + hi) / 2, (hi - lo) / 2 * 1.05
    origin = (c - h).astype(np.float32)
    spacing = (2 * h / np.array(dims)).astype(np.float32)
    wg, ig = eng.query_grid(origin, spacing, dims)
    # the same centres as explicit points: (i + 0.5) * s is exact in float64, so rounding the
    # float64 sum to float32 reproduces the kernel's single fused rounding
    ax = [(np.arange(dims[a]) + 0.5) * np.float64(spacing[a]) + np.float64(origin[a])
          for a in range(3)]
    ax = [x.astype(np.float32) for x in ax]
    Zg, Yg, Xg = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    P = torch.from_numpy(np.stack([Xg, Yg, Zg], -1).reshape(-1, 3).copy()).cuda()
    w, ins = eng.query(P)
    torch.cuda.synchronize()
    assert torch.equal(wg.reshape(-1), w)
    assert torch.equal(ig.reshape(-1), ins)
    # a closed mesh: interior voxels are inside
    assert 0.2 < float(ig.float().mean()) < 0.9


def test_grid_forest_mesh_index(torch_cuda):
    fo = W.batched_forest_workload(n_meshes=3, seed=5, f_lo=2000, f_hi=8000, q_lo=10, q_hi=20)
    forest = fwn.Forest(fo.V, fo.voff, fo.F, fo.foff)
    for m in range(3):
        Vm = fo.V[fo.voff[m]:fo.voff[m + 1]]
        single = fwn.FastWindingNumber(Vm, fo.F[fo.foff[m]:fo.foff[m + 1]])
        lo = Vm.min(0)
        sp = (Vm.max(0) - lo) / 16
        a, ia = forest.query_grid(lo, sp, (16, 16, 16), mesh=m)
        b, ib = single.query_grid(lo, sp, (16, 16, 16))
        torch_cuda.cuda.synchronize()
        assert float((a - b).abs().max()) / FOUR_PI <= 1e-6
        band = ((b / FOUR_PI) - 0.5).abs() > 1e-3
        assert torch_cuda.equal(ia[band], ib[band])


def test_orientation_criterion_finds_flipped_facets(torch_cuda):
    V, F = W.icosphere(16)
    V = V.astype(np.float32)
    ref = fwn.FastWindingNumber(V, F)
    rng = np.random.default_rng(4)
    flipped = rng.random(len(F)) < 0.1
    Fin = F.copy()
    Fin[flipped] = Fin[flipped][:, [0, 2, 1]]
    crit, flip = ref.orientation_criterion(V, Fin, eps=1e-2, threshold=0.8)
    crit, flip = crit.cpu().numpy(), flip.cpu().numpy().astype(bool)
    np.testing.assert_array_equal(flip, flipped)
    assert np.all(np.abs(np.abs(crit) - 1.0) < 0.05)
    # bad index -> INVALID_ARG
    Fb = Fin.copy()
    Fb[0, 0] = len(V) + 3
    with pytest.raises(fwn.WindingError, match="out of range"):
        ref.orientation_criterion(V, Fb)


def test_sample_inside(torch_cuda):
    V, F = W.icosphere(24)
    eng = fwn.FastWindingNumber(V.astype(np.float32), F)
    P = eng.sample_inside(200_000, seed=1)
    r = P.norm(dim=1)
    assert float(r.max()) <= 1.0 + 1e-6
    frac = P.shape[0] / 200_000  # sphere inside its bounding cube: pi/6 (minus faceting)
    assert abs(frac - math.pi / 6) < 0.01


def _grid_centres(origin, spacing, dims):
    """Voxel centres in output order (x fastest). With a dyadic origin and spacing every centre
    origin + (i + 0.5) * spacing is a float exactly, so this equals the kernel's fused form."""
    ax = []
    for a in range(3):
        x = (np.arange(dims[a]) + 0.5) * np.float64(spacing[a]) + np.float64(origin[a])
        assert np.all(x.astype(np.float32).astype(np.float64) == x)  # exact in float
        ax.append(x.astype(np.float32))
    Zg, Yg, Xg = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return np.stack([Xg, Yg, Zg], -1).reshape(-1, 3).copy()


def test_grid_matches_oracle(torch_cuda, oracle_mod):
    """The voxel sign pass against the oracle, the way volume::mesh_to_volume classifies each
    voxel centre with engine.is_inside (modules/volume/src/mesh_to_volume.cpp:167-183):
    at beta = 2, mixed vs the FP64 restatement of the same tree (O3) within 2e-6 and is_inside
    identical outside the +-1e-3 band; at beta -> infinity, vs the FP64 brute force (O1)."""
    V, F = W.displaced_icosphere(24, 1)  # 11,520 triangles, radius ~1 +- 0.16
    dims = (24, 24, 24)
    origin = np.full(3, -1.3125, np.float32)   # -21/16
    spacing = np.full(3, 0.109375, np.float32)  # 7/64: the grid spans [-1.3125, 1.3125]
    P = _grid_centres(origin, spacing, dims)
    eng = fwn.FastWindingNumber(V, F, leaf_size=8)
    wg, ig = eng.query_grid(origin, spacing, dims)
    torch_cuda.cuda.synchronize()
    wg, ig = wg.reshape(-1).cpu().numpy().astype(np.float64), ig.reshape(-1).cpu().numpy()
    o3 = oracle_mod.LbvhTree(V, F, leaf_size=8).query_f64(P, beta=2.0)
    assert np.max(np.abs(wg - o3)) / FOUR_PI <= 2e-6
    band = np.abs(o3 / FOUR_PI - 0.5) > 1e-3
    np.testing.assert_array_equal(ig[band], (o3[band] / FOUR_PI > 0.5).astype(np.uint8))
    assert 0.2 < ig.mean() < 0.8
    exact_eng = fwn.FastWindingNumber(V, F, leaf_size=8, beta=1e30)  # every leaf evaluated
    wx, ix = exact_eng.query_grid(origin, spacing, dims)
    torch_cuda.cuda.synchronize()
    wx, ix = wx.reshape(-1).cpu().numpy().astype(np.float64), ix.reshape(-1).cpu().numpy()
    o1 = oracle_mod.brute_f64(V, F, P)
    assert np.max(np.abs(wx - o1)) / FOUR_PI <= 1e-5
    band1 = np.abs(o1 / FOUR_PI - 0.5) > 1e-3
    np.testing.assert_array_equal(ix[band1], (o1[band1] / FOUR_PI > 0.5).astype(np.uint8))


def _orientation_points(V, F, eps):
    """The example's query points in float32, one operation at a time
    (modules/winding/examples/fix_orientation.cpp:93-100): n = normalized((b - a) x (c - a)),
    barycentre (a + b + c) / 3, points barycentre +- eps * n."""
    f32 = np.float32
    a, b, c = (V[F[:, j]].astype(f32) for j in range(3))
    u, v = b - a, c - a
    n = np.stack([u[:, 1] * v[:, 2] - u[:, 2] * v[:, 1],
                  u[:, 2] * v[:, 0] - u[:, 0] * v[:, 2],
                  u[:, 0] * v[:, 1] - u[:, 1] * v[:, 0]], 1).astype(f32)
    ln = np.sqrt((n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]).astype(f32)
    pos = ln > 0
    n[pos] = n[pos] / ln[pos, None]
    bary = ((a + b) + c) / f32(3)
    e = f32(eps) * n
    return (bary + e).astype(f32), (bary - e).astype(f32)


def test_orientation_criterion_matches_oracle(torch_cuda, oracle_mod):
    """fwn_orientation_criterion against the oracle's (Omega(b + eps n) - Omega(b - eps n)) / 4 pi
    (modules/winding/examples/fix_orientation.cpp:93-100) on 400 facets: at beta = 2 against the
    FP64 restatement of the same tree (O3), at beta -> infinity against the FP64 brute force (O1);
    the flip decision follows the oracle's criterion wherever it is clear of the threshold."""
    V, F = W.displaced_icosphere(12, 3)  # reference mesh
    V = V.astype(np.float32)
    rng = np.random.default_rng(9)
    pick = rng.choice(len(F), 400, replace=False)
    Fq = F[pick].copy()
    flipped = rng.random(len(Fq)) < 0.2
    Fq[flipped] = Fq[flipped][:, [0, 2, 1]]
    eps, thr = 1e-2, 0.8
    pp, pm = _orientation_points(V, Fq, eps)
    for beta, oracle_om, tol in (
            (2.0, lambda Q: oracle_mod.LbvhTree(V, F, leaf_size=8).query_f64(Q, beta=2.0), 4e-6),
            (1e30, lambda Q: oracle_mod.brute_f64(V, F, Q), 2e-5)):
        eng = fwn.FastWindingNumber(V, F, leaf_size=8, beta=beta)
        crit, flip = eng.orientation_criterion(V, Fq, eps=eps, threshold=thr)
        crit = crit.cpu().numpy().astype(np.float64)
        flip = flip.cpu().numpy().astype(bool)
        ref = (oracle_om(pp) - oracle_om(pm)) / FOUR_PI
        assert np.max(np.abs(crit - ref)) <= tol, (beta, np.max(np.abs(crit - ref)))
        clear = np.abs(ref - thr) > 1e-3
        np.testing.assert_array_equal(flip[clear], ref[clear] > thr)
        np.testing.assert_array_equal(flip, flipped)  # a closed mesh: exactly the flipped facets
