"""Autotuner (fwn_autotune): picks leaf size, schedule, block and variant by timing candidates
on the device; the tuned engine must give the same answers (within the parity tolerance) and the
cache must return the stored choice without timing."""
import math

import numpy as np
import pytest

import lagrange_gb300 as fwn
from lagrange_gb300 import workloads as W

pytestmark = pytest.mark.gpu
FOUR_PI = 4 * math.pi


def test_autotune_choice_and_cache(tmp_path):
    import torch
    torch.cuda.set_device(0)
    wl = W.displaced_icosphere_workload(nu=60, n_queries=60_000)
    cache = tmp_path / "tune.txt"
    r = fwn.autotune(wl.V, wl.F, wl.Q, cache_path=str(cache))
    assert r["from_cache"] == 0 and r["candidates"] == 108 and r["ms"] > 0  # 3 builders x 4 x 9
    assert r["leaf_size"] in (4, 8, 12, 16) and r["builder"] in (0, 1, 2)
    assert r["traversal"] in (fwn.TRAVERSAL_THREAD, fwn.TRAVERSAL_WARP)
    assert r["block_size"] % 32 == 0
    # the cached answer comes back without timing
    r2 = fwn.autotune(wl.V, wl.F, wl.Q, cache_path=str(cache))
    assert r2["from_cache"] == 1 and r2["candidates"] == 0
    assert r2["config"] == r["config"]
    assert len(cache.read_text().splitlines()) == 1
    # an entry out of range (an edited or damaged file) is ignored and the mesh tuned again
    key = cache.read_text().split()[0]
    cache.write_text(f"{key} 99 2 128 17 0 1.0\n")
    r3 = fwn.autotune(wl.V, wl.F, wl.Q, cache_path=str(cache))
    assert r3["from_cache"] == 0 and r3["candidates"] == 108 and r3["leaf_size"] in (4, 8, 12, 16)
    # the tuned engine agrees with the plain FP64 form built with the same leaf size
    eng = fwn.FastWindingNumber(wl.V, wl.F, records=fwn.RECORDS_F32 | fwn.RECORDS_F64,
                                **r["config"])
    Qd = torch.from_numpy(wl.Q).cuda()
    w, ins = eng.query(Qd)
    w64, _ = eng.query(Qd, precision=fwn.PRECISION_FP64)
    torch.cuda.synchronize()
    assert float((w.double() - w64.double()).abs().max()) / FOUR_PI <= 2e-6


def test_forest_autotune_choice_and_cache(tmp_path):
    import torch
    torch.cuda.set_device(0)
    fo = W.batched_forest_workload(n_meshes=12, seed=6, f_lo=500, f_hi=20000, q_lo=500, q_hi=20000)
    cache = tmp_path / "tune_forest.txt"
    r = fwn.autotune_forest(fo.V, fo.voff, fo.F, fo.foff, fo.Q, fo.qoff, cache_path=str(cache))
    assert r["from_cache"] == 0 and r["candidates"] == 40 and r["ms"] > 0  # 2 builders x 4 x 5
    assert r["builder"] in (0, 1)
    assert r["tuning"] in (1, 3, 4, 5, 6)
    assert r["leaf_size"] in (4, 8, 12, 16) and r["traversal"] == fwn.TRAVERSAL_WARP
    r2 = fwn.autotune_forest(fo.V, fo.voff, fo.F, fo.foff, fo.Q, fo.qoff, cache_path=str(cache))
    assert r2["from_cache"] == 1 and r2["config"] == r["config"]
    # the chosen forest agrees with its FP64 form
    forest = fwn.Forest(fo.V, fo.voff, fo.F, fo.foff, records=fwn.RECORDS_F32 | fwn.RECORDS_F64,
                        **r["config"])
    Qd = torch.from_numpy(fo.Q).cuda()
    w, _ = forest.query_forest(Qd, fo.qoff)
    w64, _ = forest.query_forest(Qd, fo.qoff, precision=fwn.PRECISION_FP64)
    torch.cuda.synchronize()
    assert float((w.double() - w64.double()).abs().max()) / FOUR_PI <= 2e-6
    # invalid offsets are refused
    bad = fo.qoff.copy()
    bad[1], bad[2] = bad[2], bad[1]
    if bad[1] != bad[2]:
        with pytest.raises(fwn.WindingError, match="non-decreasing"):
            fwn.autotune_forest(fo.V, fo.voff, fo.F, fo.foff, fo.Q, bad)
