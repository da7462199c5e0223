"""Queries split across several GPUs (one process per GPU), each holding a replica of the tree.

The reference answers one point per call on one host (modules/winding/src/FastWindingNumber.cpp:
60-76); its only concurrency is the per-voxel callback from OpenVDB's worker threads
(modules/volume/src/mesh_to_volume.cpp:175-183). Queries are independent given the tree, so the
path shards with no collective during compute:

* one mesh: every rank builds (or holds) a replica of the tree and computes the same Hilbert-curve
  order of the whole point set (the permutation the query applies itself); rank r answers the
  r-th contiguous range of that order, so each rank's points form one compact region of space
  and its warps stay as coherent as on one GPU. One all-gather then returns every rank's Omega
  and inside, which are scattered back to the caller's order.
* a forest: whole meshes are assigned to ranks by LPT bin packing on the estimated cost
  Q * log2(F + 1) (largest first, each to the least loaded rank); each rank builds and queries
  only its meshes.

The split and gather logic is plain array code (numpy or torch), independent of how a shard is
evaluated, so it is tested on CPU ranks with the oracle as the evaluator; on GPUs the evaluator
is the engine's query and the collective is NCCL's all-gather.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np


def shard_ranges(n: int, world: int) -> list[tuple[int, int]]:
    """Contiguous ranges [start, end) of n sorted points, one per rank, sizes differing by <= 1
    (the first n % world ranks take one more)."""
    if world < 1 or n < 0:
        raise ValueError("world must be >= 1 and n >= 0")
    base, extra = divmod(n, world)
    out, s = [], 0
    for r in range(world):
        e = s + base + (1 if r < extra else 0)
        out.append((s, e))
        s = e
    return out


def lpt_assign(costs: Sequence[float], world: int) -> list[list[int]]:
    """Longest-processing-time bin packing: items by decreasing cost (ties by index), each to the
    rank with the smallest load so far (ties to the lowest rank). Returns each rank's item
    indices in increasing order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    bins: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        bins[r].append(i)
        load[r] += float(costs[i])
    return [sorted(b) for b in bins]


def forest_costs(triangle_offsets, query_offsets) -> np.ndarray:
    """Estimated query cost per mesh of a forest: Q * log2(F + 1)."""
    f = np.diff(np.asarray(triangle_offsets, np.int64)).astype(np.float64)
    q = np.diff(np.asarray(query_offsets, np.int64)).astype(np.float64)
    return q * np.log2(f + 1.0)


def _cat(xs):
    if isinstance(xs[0], np.ndarray):
        return np.concatenate(xs)
    import torch
    return torch.cat(xs)


def gather_sharded(order, parts: Sequence, n: int):
    """Reassembles per-rank results into the caller's order: parts[r] holds the results of the
    points order[start_r:end_r] (shard_ranges(n, world)), so out[order[k]] = concat(parts)[k]."""
    full = _cat(list(parts))
    if len(full) != n:
        raise ValueError("the parts do not cover the point set")
    if isinstance(full, np.ndarray):
        out = np.empty_like(full)
        out[np.asarray(order)] = full
        return out
    import torch
    idx = torch.as_tensor(np.asarray(order) if isinstance(order, np.ndarray) else order,
                          device=full.device).long()
    out = full.new_empty(full.shape)
    out[idx] = full
    return out


def query_sharded(points, order, rank: int, world: int,
                  evaluate: Callable, all_gather: Callable):
    """One mesh, `world` ranks: this rank evaluates its contiguous range of `order` (the
    Hilbert-curve order of all points, the same on every rank) with `evaluate(points_subset)` ->
    (omega, inside); `all_gather(x)` returns the list of every rank's x (rank order). Returns
    (omega, inside) of all points in the caller's order, on every rank."""
    n = len(points)
    start, end = shard_ranges(n, world)[rank]
    idx = order[start:end]
    omega, inside = evaluate(points[idx])
    return (gather_sharded(order, all_gather(omega), n),
            gather_sharded(order, all_gather(inside), n))


def torch_all_gather(dist, group=None) -> Callable:
    """all_gather over torch.distributed for shards whose lengths differ by at most one: pads to
    the longest shard, gathers, and trims each part back to its own length."""
    def gather(x):
        import torch
        world = dist.get_world_size(group)
        n_local = torch.tensor([x.shape[0]], dtype=torch.int64, device=x.device)
        sizes = [torch.zeros_like(n_local) for _ in range(world)]
        dist.all_gather(sizes, n_local, group=group)
        m = int(max(int(s.item()) for s in sizes))
        buf = x.new_zeros((m,) + tuple(x.shape[1:]))
        buf[: x.shape[0]] = x
        parts = [x.new_empty(buf.shape) for _ in range(world)]
        dist.all_gather(parts, buf, group=group)
        return [p[: int(s.item())] for p, s in zip(parts, sizes)]
    return gather


def engine_query_sharded(engine, points, dist, group=None, stream=None):
    """fwn on several GPUs: `engine` is this rank's replica of the same mesh, `points` the whole
    point set (CUDA tensor, identical on every rank). Every rank computes the query order of
    all points, answers its contiguous range of it (already sorted, so queried with
    sort_queries=0), and one all-gather returns the results to every rank in the caller's order.
    Returns (omega float32, inside uint8) CUDA tensors."""
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    order = engine.query_order(points, stream=stream)

    def evaluate(sub):
        return engine.query(sub.contiguous(), sort_queries=False, stream=stream)

    return query_sharded(points, order, rank, world, evaluate, torch_all_gather(dist, group))


def forest_shard(voff, foff, qoff, rank: int, world: int):
    """The meshes a rank builds and queries (LPT on Q * log2(F + 1)) and the sub-forest's offsets:
    returns (meshes, vertex ranges, triangle ranges, query ranges, sub_voff, sub_foff, sub_qoff),
    ranges as (start, end) into the full arrays."""
    meshes = lpt_assign(forest_costs(foff, qoff), world)[rank]
    vr = [(int(voff[m]), int(voff[m + 1])) for m in meshes]
    fr = [(int(foff[m]), int(foff[m + 1])) for m in meshes]
    qr = [(int(qoff[m]), int(qoff[m + 1])) for m in meshes]

    def offs(rs):
        return np.concatenate([[0], np.cumsum([e - s for s, e in rs])]).astype(np.int64)
    return meshes, vr, fr, qr, offs(vr), offs(fr), offs(qr)


def gather_forest(qoff, shards: Sequence, parts: Sequence):
    """Reassembles per-rank forest results: shards[r] = forest_shard(...)[3] (rank r's query
    ranges, in its sub-forest's order) and parts[r] its results; returns the full array in the
    forest's query order."""
    n = int(np.asarray(qoff)[-1])
    out = None
    for ranges, part in zip(shards, parts):
        if out is None:
            out = np.empty(n, dtype=np.asarray(part).dtype) if isinstance(part, np.ndarray) \
                else part.new_empty((n,))
        k = 0
        for s, e in ranges:
            out[s:e] = part[k:k + (e - s)]
            k += e - s
        if k != len(part):
            raise ValueError("a rank's part does not match its query ranges")
    return out


__all__ = ["shard_ranges", "lpt_assign", "forest_costs", "gather_sharded", "query_sharded",
           "torch_all_gather", "engine_query_sharded", "forest_shard", "gather_forest"]
