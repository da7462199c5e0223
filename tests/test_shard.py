"""Queries split across ranks (lagrange_gb300.shard): the split and gather logic on CPU, and a
two-rank gloo run whose ranks evaluate their shards with the CPU oracle and gather the results,
checked bit for bit against a single-rank oracle run over all points.

One mesh: every rank holds the same tree and the same query order; rank r answers the r-th
contiguous range of that order. A forest: whole meshes go to ranks by LPT bin packing on
Q * log2(F + 1). Nothing here needs a GPU."""
import json
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

from lagrange_gb300 import shard
from lagrange_gb300 import workloads as W

ROOT = Path(__file__).resolve().parent.parent
FOUR_PI = 4 * np.pi


def test_shard_ranges_cover_in_order():
    for n in (0, 1, 7, 10, 1001):
        for world in (1, 2, 3, 8):
            r = shard.shard_ranges(n, world)
            assert len(r) == world and r[0][0] == 0 and r[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
            sizes = [e - s for s, e in r]
            assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)
    with pytest.raises(ValueError):
        shard.shard_ranges(5, 0)


def test_lpt_assign_balances_and_covers():
    rng = np.random.default_rng(0)
    costs = rng.lognormal(0, 1.5, 200)
    for world in (1, 2, 3, 8):
        bins = shard.lpt_assign(costs, world)
        items = sorted(i for b in bins for i in b)
        assert items == list(range(len(costs)))
        loads = [costs[b].sum() for b in bins]
        # LPT: the spread of the loads is at most the largest single item
        assert max(loads) - min(loads) <= costs.max() + 1e-9
    assert shard.lpt_assign([5, 1, 1, 1, 1, 1], 2) == [[0], [1, 2, 3, 4, 5]]


def test_gather_sharded_round_trip():
    rng = np.random.default_rng(1)
    n, world = 1003, 3
    order = rng.permutation(n)
    vals = rng.normal(size=n)
    parts = [vals[order[s:e]] for s, e in shard.shard_ranges(n, world)]
    np.testing.assert_array_equal(shard.gather_sharded(order, parts, n), vals)
    with pytest.raises(ValueError):
        shard.gather_sharded(order, parts[:2], n)


def test_forest_shard_and_gather_with_empty_meshes():
    """Meshes without triangles or without queries (and more ranks than meshes with work) are
    assigned and gathered like any other: every query lands back at its own offset."""
    foff = np.array([0, 10, 10, 40, 40, 41, 100], np.int64)       # meshes 1 and 3 empty
    voff = np.array([0, 12, 12, 50, 50, 53, 130], np.int64)
    qoff = np.array([0, 5, 9, 9, 12, 12, 30], np.int64)            # meshes 2 and 4 no queries
    vals = np.arange(qoff[-1], dtype=np.float64) * 1.5
    for world in (1, 2, 4, 9):
        shards = [shard.forest_shard(voff, foff, qoff, r, world) for r in range(world)]
        assigned = sorted(m for sh in shards for m in sh[0])
        assert assigned == list(range(len(foff) - 1))
        parts = []
        for meshes, vr, fr, qr, svoff, sfoff, sqoff in shards:
            assert len(svoff) == len(meshes) + 1 and svoff[-1] == sum(e - s for s, e in vr)
            assert sfoff[-1] == sum(e - s for s, e in fr) and sqoff[-1] == sum(e - s for s, e in qr)
            parts.append(np.concatenate([vals[s:e] for s, e in qr]) if qr else np.zeros(0))
        np.testing.assert_array_equal(shard.gather_forest(qoff, [sh[3] for sh in shards], parts),
                                      vals)


def _morton_order(P):
    """A spatially coherent order of the points (Morton code on a 1024^3 grid): stands in for the
    device's Hilbert order, which every rank computes the same way."""
    lo, hi = P.min(0), P.max(0)
    c = np.clip(((P - lo) / np.maximum(hi - lo, 1e-30) * 1023).astype(np.int64), 0, 1023)
    code = np.zeros(len(P), np.int64)
    for b in range(10):
        for a in range(3):
            code |= ((c[:, a] >> b) & 1) << (3 * b + a)
    return np.argsort(code, kind="stable")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, outdir):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import oracle
    from lagrange_gb300 import shard as S
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    gather = S.torch_all_gather(dist)
    # one mesh, contiguous ranges of the query order
    wl = W.displaced_icosphere_workload(nu=12, n_queries=3001)
    tree = oracle.LbvhTree(wl.V, wl.F, leaf_size=8)
    order = _morton_order(wl.Q)

    def evaluate(sub):
        om = tree.query_f64(sub, beta=2.0)
        return torch.from_numpy(om), torch.from_numpy((om / FOUR_PI > 0.5).astype(np.uint8))
    om, ins = S.query_sharded(wl.Q, order, rank, world, evaluate, gather)
    np.save(Path(outdir) / f"mesh_om_{rank}.npy", om.numpy())
    np.save(Path(outdir) / f"mesh_in_{rank}.npy", ins.numpy())
    # a forest: whole meshes per rank (LPT), each rank building only its meshes
    fo = W.batched_forest_workload(n_meshes=7, seed=11, f_lo=200, f_hi=3000, q_lo=50, q_hi=900)
    meshes, vr, fr, qr, _, _, _ = S.forest_shard(fo.voff, fo.foff, fo.qoff, rank, world)
    mine = []
    for m, (v0, v1), (f0, f1), (q0, q1) in zip(meshes, vr, fr, qr):
        t = oracle.LbvhTree(fo.V[v0:v1], fo.F[f0:f1], leaf_size=8)
        mine.append(t.query_f64(fo.Q[q0:q1], beta=2.0))
    part = np.concatenate(mine) if mine else np.zeros(0)
    parts = gather(torch.from_numpy(part))
    shards = [S.forest_shard(fo.voff, fo.foff, fo.qoff, r, world)[3] for r in range(world)]
    full = S.gather_forest(fo.qoff, shards, parts)
    np.save(Path(outdir) / f"forest_{rank}.npy", full.numpy())
    (Path(outdir) / f"meshes_{rank}.json").write_text(json.dumps(meshes))
    dist.destroy_process_group()


def test_two_gloo_ranks_split_and_gather_match_single_rank(tmp_path):
    import torch.multiprocessing as mp
    sys.path.insert(0, str(ROOT))
    import oracle
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    # single-rank oracle runs over all points
    wl = W.displaced_icosphere_workload(nu=12, n_queries=3001)
    ref = oracle.LbvhTree(wl.V, wl.F, leaf_size=8).query_f64(wl.Q, beta=2.0)
    for r in range(world):
        np.testing.assert_array_equal(np.load(tmp_path / f"mesh_om_{r}.npy"), ref)
        np.testing.assert_array_equal(np.load(tmp_path / f"mesh_in_{r}.npy"),
                                      (ref / FOUR_PI > 0.5).astype(np.uint8))
    fo = W.batched_forest_workload(n_meshes=7, seed=11, f_lo=200, f_hi=3000, q_lo=50, q_hi=900)
    fref = np.concatenate([
        oracle.LbvhTree(fo.V[fo.voff[m]:fo.voff[m + 1]], fo.F[fo.foff[m]:fo.foff[m + 1]],
                        leaf_size=8).query_f64(fo.Q[fo.qoff[m]:fo.qoff[m + 1]], beta=2.0)
        for m in range(7)])
    owned = []
    for r in range(world):
        np.testing.assert_array_equal(np.load(tmp_path / f"forest_{r}.npy"), fref)
        owned += json.loads((tmp_path / f"meshes_{r}.json").read_text())
    assert sorted(owned) == list(range(7))  # every mesh on exactly one rank
