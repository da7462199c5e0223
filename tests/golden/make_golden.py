"""Generates the golden fixtures in this folder (run from the repo root:
``python tests/golden/make_golden.py``).

The reference path cannot be built or imported here (its arithmetic is in the absent
third-party library jdumas/WindingNumber@a48b8f55; its tests pin no values), so the fixtures
are produced by the oracle and by closed-form solid angles:

* ``analytic.npz``    closed-form solid angles (octant triangle, square seen from its axis,
                      degenerate triangle, query on a vertex) — these pin the oracle itself.
* ``triangles.npz``   64 random triangles, one query each, FP64 oracle solid angle.
* ``uv_sphere.npz``   the 64x32 UV sphere, its first 4,096 seed-0 queries, the FP64
                      brute-force solid angle (O1), the FP64 LBVH value at beta=2, leaf 4 (O3)
                      and the reference-restatement is_inside (O2).
* ``displaced.npz``   displaced icosphere frequency 24 (11,520 triangles, seed 1) with 1,024
                      box and 1,024 near-surface queries and their O1 solid angles.
* ``soup.npz``        the defective soup at frequency 20 (10% of the faces deleted, 1% flipped,
                      0.5% duplicated with 1e-7 jitter), 1,024 box and 1,024 near-surface
                      (within 1e-4) queries: O1, O3 at beta=2 leaf 8, and O2's is_inside.
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from lagrange_gb300 import workloads as W  # noqa: E402


def analytic():
    tris, qs, om = [], [], []
    # octant triangle seen from the origin: 4 pi / 8
    tris.append([[1, 0, 0], [0, 1, 0], [0, 0, 1]]); qs.append([0, 0, 0]); om.append(math.pi / 2)
    # reversed: -pi/2
    tris.append([[1, 0, 0], [0, 0, 1], [0, 1, 0]]); qs.append([0, 0, 0]); om.append(-math.pi / 2)
    # square [-1,1]^2 at z=0 (normal +z) seen from (0,0,-h): 4 asin(a b / sqrt((a2+h2)(b2+h2)))
    for h in (0.5, 1.0, 2.0):
        val = 4 * math.asin(1.0 / math.sqrt((1 + h * h) * (1 + h * h)))
        # two triangles; the fixture stores the pair's sum on the first, 0 target on the second
        tris.append([[-1, -1, 0], [1, -1, 0], [1, 1, 0]]); qs.append([0, 0, -h])
        tris.append([[-1, -1, 0], [1, 1, 0], [-1, 1, 0]]); qs.append([0, 0, -h])
        om.append(val); om.append(np.nan)  # NaN: covered by the pair sum
    # degenerate (collinear) triangle: 0
    tris.append([[0, 0, 0], [1, 1, 1], [2, 2, 2]]); qs.append([0.3, -0.2, 0.9]); om.append(0.0)
    # query exactly on a vertex: 0 (finite)
    tris.append([[0, 0, 0], [1, 0, 0], [0, 1, 0]]); qs.append([1, 0, 0]); om.append(0.0)
    # query in the plane outside the triangle: 0
    tris.append([[0, 0, 0], [1, 0, 0], [0, 1, 0]]); qs.append([2, 2, 0]); om.append(0.0)
    return (np.array(tris, np.float64), np.array(qs, np.float64), np.array(om, np.float64))


def main():
    oracle.build()
    rng = np.random.default_rng(12345)
    T, Qa, Oa = analytic()
    np.savez_compressed(HERE / "analytic.npz", tris=T, queries=Qa, omega=Oa)

    tri = rng.uniform(-1, 1, (64, 3, 3)).astype(np.float32)
    q = rng.uniform(-1.5, 1.5, (64, 3)).astype(np.float32)
    om = np.array([oracle.tri_solid_angle(t[0], t[1], t[2], p) for t, p in zip(tri, q)])
    np.savez_compressed(HERE / "triangles.npz", tris=tri, queries=q, omega=om)

    wl = W.uv_sphere_workload(4096)
    o1 = oracle.brute_f64(wl.V, wl.F, wl.Q)
    o3 = oracle.LbvhTree(wl.V, wl.F, leaf_size=4).query_f64(wl.Q, beta=2.0)
    _, ins = oracle.RefTree(wl.V, wl.F, 4).query(wl.Q, beta=2.0)
    np.savez_compressed(HERE / "uv_sphere.npz", V=wl.V, F=wl.F, Q=wl.Q, omega_exact=o1,
                        omega_lbvh_beta2=o3, inside_ref=ins)

    d = W.displaced_icosphere_workload(nu=24, n_queries=2048)
    o1 = oracle.brute_f64(d.V, d.F, d.Q)
    np.savez_compressed(HERE / "displaced.npz", V=d.V, F=d.F, Q=d.Q, near=d.near_mask,
                        omega_exact=o1)
    sp = W.defective_soup_workload(nu=20, n_queries=2048)
    o1 = oracle.brute_f64(sp.V, sp.F, sp.Q)
    o3 = oracle.LbvhTree(sp.V, sp.F, leaf_size=8).query_f64(sp.Q, beta=2.0)
    _, ins = oracle.RefTree(sp.V, sp.F, 8).query(sp.Q, beta=2.0)
    np.savez_compressed(HERE / "soup.npz", V=sp.V, F=sp.F, Q=sp.Q, near=sp.near_mask,
                        omega_exact=o1, omega_lbvh_beta2=o3, inside_ref=ins)
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
