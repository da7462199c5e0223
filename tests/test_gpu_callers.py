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
