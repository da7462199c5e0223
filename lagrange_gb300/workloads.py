"""Seeded synthetic meshes and query sets for the fast-winding-number workloads.

The reference benchmark (modules/winding/tests/test_fast_winding_number.cpp:85-125) uses
``open/core/dragon.obj`` from an external data repository that is not available; these
generators stand in for it with closed, open and batched meshes of the sizes and value
distributions of the five workloads below (all float32 vertices, int32 triangles, outward CCW
winding):

1. ``uv_sphere_workload``    UV sphere r=1, 64x32 segments (3,968 tris), 100k queries U[-1.5,1.5]^3,
                             seed 0.
2. ``displaced_icosphere_workload`` geodesic icosphere frequency 316 (1,997,120 tris) radially
                             displaced by r = 1 + sum_k a_k sin(f_k (d_k . v) + phi_k), seed 1;
                             10M queries: 5M uniform in bbox*1.2, 5M on the surface offset along
                             the normal by +-U(1e-6, 1e-3).
3. ``defective_soup_workload`` the displaced icosphere at frequency 224 (1,003,520 tris), seed 2:
                             10% faces deleted, 1% flipped, 0.5% duplicated with 1e-7 jitter; 5M
                             queries, half uniform, half within 1e-4 of the surface.
4. ``batched_forest_workload`` 512 spheres / tori (R/r ~ U(2,5)), F log-uniform [1k, 500k],
                             Q log-uniform [1k, 1M], seed 3.
5. ``voxel_workload``        4 displaced icospheres of 5M tris (seeds 4-7), each queried on a 256^3
                             voxel-centre grid over bbox*1.05.

Generation uses numpy's PCG64 (``default_rng``), so the same seed gives the same arrays on every
machine.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# --------------------------------------------------------------------------------------------
# Base meshes
# --------------------------------------------------------------------------------------------


def uv_sphere(n_lon: int = 64, n_lat: int = 32, radius: float = 1.0):
    """UV sphere with n_lon segments and n_lat rings: 2 + (n_lat-1)*n_lon vertices,
    2*n_lon*(n_lat-1) triangles, outward CCW."""
    th = np.pi * np.arange(1, n_lat) / n_lat              # polar angles of the rings
    ph = 2 * np.pi * np.arange(n_lon) / n_lon
    st, ct = np.sin(th)[:, None], np.cos(th)[:, None]
    ring = np.stack([st * np.cos(ph)[None, :], st * np.sin(ph)[None, :],
                     np.broadcast_to(ct, (n_lat - 1, n_lon))], axis=-1).reshape(-1, 3)
    V = np.concatenate([[[0.0, 0.0, 1.0]], ring, [[0.0, 0.0, -1.0]]]) * radius
    north, south = 0, 1 + (n_lat - 1) * n_lon
    idx = lambda r, c: 1 + r * n_lon + (c % n_lon)  # noqa: E731
    c = np.arange(n_lon)
    tris = [np.stack([np.full(n_lon, north), idx(0, c), idx(0, c + 1)], 1)]
    for r in range(n_lat - 2):
        a, b = idx(r, c), idx(r, c + 1)
        d, e = idx(r + 1, c), idx(r + 1, c + 1)
        tris.append(np.stack([a, d, e], 1))
        tris.append(np.stack([a, e, b], 1))
    tris.append(np.stack([idx(n_lat - 2, c), np.full(n_lon, south), idx(n_lat - 2, c + 1)], 1))
    F = np.concatenate(tris).astype(np.int32)
    return V.astype(np.float32), F


def _icosahedron():
    t = (1.0 + 5 ** 0.5) / 2.0
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return V, F


def icosphere(nu: int):
    """Class-I geodesic sphere of frequency nu: 20 nu^2 triangles, 10 nu^2 + 2 shared vertices
    (unit directions, float64), outward CCW."""
    assert nu >= 1
    V0, F0 = _icosahedron()
    # canonical edges
    edges = {}
    for f in F0:
        for a, b in ((f[0], f[1]), (f[1], f[2]), (f[2], f[0])):
            key = (min(a, b), max(a, b))
            if key not in edges:
                edges[key] = len(edges)
    ne = len(edges)
    assert ne == 30
    n_int = (nu - 1) * (nu - 2) // 2
    nv = 12 + ne * (nu - 1) + 20 * n_int
    P = np.empty((nv, 3), np.float64)
    P[:12] = V0
    k = np.arange(1, nu)
    for (u, v), e in edges.items():
        pts = ((nu - k)[:, None] * V0[u] + k[:, None] * V0[v]) / nu
        P[12 + e * (nu - 1): 12 + (e + 1) * (nu - 1)] = pts
    # local grid (i, j), i + j <= nu ; point = ((nu-i-j) A + i B + j C)/nu
    ii, jj = np.meshgrid(np.arange(nu + 1), np.arange(nu + 1), indexing="ij")
    m = (ii + jj) <= nu
    gi, gj = ii[m], jj[m]
    lid = -np.ones((nu + 1, nu + 1), np.int64)
    lid[gi, gj] = np.arange(len(gi))
    interior = (gi > 0) & (gj > 0) & (gi + gj < nu)
    int_rank = -np.ones(len(gi), np.int64)
    int_rank[interior] = np.arange(interior.sum())
    # triangles in local ids
    up_i, up_j = np.nonzero((ii + jj) < nu)
    dn_i, dn_j = np.nonzero((ii + jj) < nu - 1)
    tri_local = np.concatenate([
        np.stack([lid[up_i, up_j], lid[up_i + 1, up_j], lid[up_i, up_j + 1]], 1),
        np.stack([lid[dn_i + 1, dn_j], lid[dn_i + 1, dn_j + 1], lid[dn_i, dn_j + 1]], 1)])
    Fout = np.empty((20 * nu * nu, 3), np.int64)
    for fi, (A, B, Cc) in enumerate(F0):
        gid = np.empty(len(gi), np.int64)
        # corners
        gid[(gi == 0) & (gj == 0)] = A
        gid[(gi == nu) & (gj == 0)] = B
        gid[(gi == 0) & (gj == nu)] = Cc

        def edge_ids(p, q, t):  # points at parameter t/nu from p to q
            e = edges[(min(p, q), max(p, q))]
            kk = t if p < q else nu - t
            return 12 + e * (nu - 1) + (kk - 1)

        s = (gj == 0) & (gi > 0) & (gi < nu)          # A -> B, param i
        gid[s] = edge_ids(A, B, gi[s])
        s = (gi == 0) & (gj > 0) & (gj < nu)          # A -> C, param j
        gid[s] = edge_ids(A, Cc, gj[s])
        s = (gi + gj == nu) & (gi > 0) & (gj > 0)     # B -> C, param j
        gid[s] = edge_ids(B, Cc, gj[s])
        base = 12 + ne * (nu - 1) + fi * n_int
        gid[interior] = base + int_rank[interior]
        if n_int:
            w = ((nu - gi - gj)[interior, None] * V0[A] + gi[interior, None] * V0[B] +
                 gj[interior, None] * V0[Cc]) / nu
            P[base: base + n_int] = w
        Fout[fi * nu * nu:(fi + 1) * nu * nu] = gid[tri_local]
    P /= np.linalg.norm(P, axis=1, keepdims=True)
    return P, Fout.astype(np.int32)


def torus_grid(nu_: int, nv_: int, R: float, r: float):
    """Torus as a nu_ x nv_ grid (2 nu_ nv_ triangles), outward CCW. Returns vertices, triangles,
    per-vertex unit tube normals."""
    u = 2 * np.pi * np.arange(nu_) / nu_
    v = 2 * np.pi * np.arange(nv_) / nv_
    U, W = np.meshgrid(u, v, indexing="ij")
    n = np.stack([np.cos(U) * np.cos(W), np.sin(U) * np.cos(W), np.sin(W)], -1).reshape(-1, 3)
    c = np.stack([R * np.cos(U), R * np.sin(U), np.zeros_like(U)], -1).reshape(-1, 3)
    P = c + r * n
    a = np.arange(nu_)[:, None]
    b = np.arange(nv_)[None, :]
    i00 = (a * nv_ + b)
    i10 = (((a + 1) % nu_) * nv_ + b)
    i01 = (a * nv_ + (b + 1) % nv_)
    i11 = (((a + 1) % nu_) * nv_ + (b + 1) % nv_)
    F = np.concatenate([np.stack([i00, i10, i11], -1).reshape(-1, 3),
                        np.stack([i00, i11, i01], -1).reshape(-1, 3)])
    return P, F.astype(np.int32), n, c


@dataclass
class Displacement:
    a: np.ndarray
    f: np.ndarray
    d: np.ndarray
    phi: np.ndarray

    @staticmethod
    def draw(rng: np.random.Generator, k: int = 8) -> "Displacement":
        a = rng.uniform(0.0, 0.02, k)
        f = rng.uniform(2.0, 12.0, k)
        d = rng.normal(size=(k, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        phi = rng.uniform(0.0, 2 * np.pi, k)
        return Displacement(a, f, d, phi)

    def __call__(self, unit_dirs: np.ndarray) -> np.ndarray:
        s = np.zeros(len(unit_dirs))
        for ak, fk, dk, pk in zip(self.a, self.f, self.d, self.phi):
            s += ak * np.sin(fk * (unit_dirs @ dk) + pk)
        return s


def displaced_icosphere(nu: int, seed: int):
    """Icosphere of frequency nu, radially displaced by 1 + sum_k a_k sin(f_k (d_k.v) + phi_k)
    with parameters drawn from default_rng(seed). float32 vertices."""
    rng = np.random.default_rng(seed)
    disp = Displacement.draw(rng)
    P, F = icosphere(nu)
    Vd = P * (1.0 + disp(P))[:, None]
    return Vd.astype(np.float32), F


# --------------------------------------------------------------------------------------------
# Query generators
# --------------------------------------------------------------------------------------------


def box_queries(V: np.ndarray, n: int, rng: np.random.Generator, scale: float = 1.2):
    lo, hi = V.min(0).astype(np.float64), V.max(0).astype(np.float64)
    c, h = (lo + hi) / 2, (hi - lo) / 2 * scale
    return (c + rng.uniform(-1.0, 1.0, (n, 3)) * h).astype(np.float32)


def surface_queries(V: np.ndarray, F: np.ndarray, n: int, rng: np.random.Generator,
                    off_lo: float, off_hi: float):
    """Points on random triangles (area-weighted, uniform barycentrics) offset along the unit
    normal by +-U(off_lo, off_hi)."""
    Vd = V.astype(np.float64)
    a, b, c = Vd[F[:, 0]], Vd[F[:, 1]], Vd[F[:, 2]]
    nrm = np.cross(b - a, c - a)
    area = np.linalg.norm(nrm, axis=1)
    cdf = np.cumsum(area)
    t = np.searchsorted(cdf, rng.uniform(0.0, cdf[-1], n), side="right")
    t = np.minimum(t, len(F) - 1)
    r1, r2 = rng.uniform(size=n), rng.uniform(size=n)
    s1 = np.sqrt(r1)
    w0, w1, w2 = 1 - s1, s1 * (1 - r2), s1 * r2
    p = w0[:, None] * a[t] + w1[:, None] * b[t] + w2[:, None] * c[t]
    un = nrm[t] / np.maximum(area[t], 1e-300)[:, None]
    sign = np.where(rng.uniform(size=n) < 0.5, -1.0, 1.0)
    off = sign * rng.uniform(off_lo, off_hi, n)
    return (p + off[:, None] * un).astype(np.float32)


# --------------------------------------------------------------------------------------------
# Workloads
# --------------------------------------------------------------------------------------------


@dataclass
class Workload:
    name: str
    V: np.ndarray
    F: np.ndarray
    Q: np.ndarray
    beta: float = 2.0
    near_mask: np.ndarray | None = None  # queries placed close to the surface
    meta: dict = field(default_factory=dict)


def uv_sphere_workload(n_queries: int = 100_000, seed: int = 0) -> Workload:
    V, F = uv_sphere(64, 32)
    rng = np.random.default_rng(seed)
    Q = rng.uniform(-1.5, 1.5, (n_queries, 3)).astype(np.float32)
    return Workload("uv_sphere_64x32_q100k", V, F, Q,
                    meta=dict(triangles=len(F), queries=len(Q)))


def displaced_icosphere_workload(nu: int = 316, n_queries: int = 10_000_000, seed: int = 1,
                                 near_lo: float = 1e-6, near_hi: float = 1e-3) -> Workload:
    V, F = displaced_icosphere(nu, seed)
    rng = np.random.default_rng(seed + 1000)
    nb = n_queries // 2
    Qb = box_queries(V, nb, rng, 1.2)
    Qs = surface_queries(V, F, n_queries - nb, rng, near_lo, near_hi)
    Q = np.concatenate([Qb, Qs])
    near = np.zeros(len(Q), bool)
    near[nb:] = True
    return Workload(f"displaced_icosphere_nu{nu}_q{n_queries}", V, F, Q, near_mask=near,
                    meta=dict(triangles=len(F), queries=len(Q), nu=nu, seed=seed))


def defective_soup_workload(nu: int = 224, n_queries: int = 5_000_000, seed: int = 2) -> Workload:
    V, F = displaced_icosphere(nu, 1)  # the displaced icosphere's surface, at frequency nu
    rng = np.random.default_rng(seed)
    nf = len(F)
    keep = rng.permutation(nf)[: nf - nf // 10]  # delete 10%
    keep.sort()
    F = F[keep].copy()
    nf = len(F)
    flip = rng.choice(nf, nf // 100, replace=False)
    F[flip] = F[flip][:, [0, 2, 1]]
    dup = rng.choice(nf, nf // 200, replace=False)
    newv = V[F[dup].reshape(-1)].astype(np.float64)
    newv += rng.uniform(-1e-7, 1e-7, newv.shape)
    base = len(V)
    V = np.concatenate([V, newv.astype(np.float32)])
    Fd = (base + np.arange(3 * len(dup))).reshape(-1, 3).astype(np.int32)
    F = np.concatenate([F, Fd]).astype(np.int32)
    qrng = np.random.default_rng(seed + 1000)
    nb = n_queries // 2
    Q = np.concatenate([box_queries(V, nb, qrng, 1.2),
                        surface_queries(V, F, n_queries - nb, qrng, 0.0, 1e-4)])
    near = np.zeros(len(Q), bool)
    near[nb:] = True
    return Workload(f"defective_soup_nu{nu}_q{n_queries}", V, F, Q, near_mask=near,
                    meta=dict(triangles=len(F), queries=len(Q), nu=nu, seed=seed))


@dataclass
class Forest:
    name: str
    V: np.ndarray
    F: np.ndarray           # local indices per mesh
    voff: np.ndarray        # int64 [M+1]
    foff: np.ndarray
    Q: np.ndarray
    qoff: np.ndarray
    beta: float = 2.0
    meta: dict = field(default_factory=dict)


def _sphere_for(nf_target: int, rng):
    nu = max(7, int(round(math.sqrt(nf_target / 20.0))))
    P, F = icosphere(nu)
    disp = Displacement.draw(rng)
    V = P * (1.0 + disp(P))[:, None]
    return V.astype(np.float32), F


def _torus_for(nf_target: int, rng):
    ratio = rng.uniform(2.0, 5.0)
    R, r = 1.0, 1.0 / ratio
    nv_ = max(6, int(round(math.sqrt(nf_target / (2.0 * ratio)))))
    nu_ = max(6, int(round(nf_target / (2.0 * nv_))))
    P, F, n, c = torus_grid(nu_, nv_, R, r)
    disp = Displacement.draw(rng)
    V = c + (r * (1.0 + disp(n)))[:, None] * n
    return V.astype(np.float32), F


def batched_forest_workload(n_meshes: int = 512, seed: int = 3, f_lo: int = 1000,
                            f_hi: int = 500_000, q_lo: int = 1000, q_hi: int = 1_000_000) -> Forest:
    rng = np.random.default_rng(seed)
    Vs, Fs, Qs = [], [], []
    for m in range(n_meshes):
        nf = int(round(math.exp(rng.uniform(math.log(f_lo), math.log(f_hi)))))
        nq = int(round(math.exp(rng.uniform(math.log(q_lo), math.log(q_hi)))))
        V, F = (_sphere_for if rng.uniform() < 0.5 else _torus_for)(nf, rng)
        Vs.append(V)
        Fs.append(F)
        Qs.append(box_queries(V, nq, rng, 1.2))
    voff = np.concatenate([[0], np.cumsum([len(v) for v in Vs])]).astype(np.int64)
    foff = np.concatenate([[0], np.cumsum([len(f) for f in Fs])]).astype(np.int64)
    qoff = np.concatenate([[0], np.cumsum([len(q) for q in Qs])]).astype(np.int64)
    return Forest(f"forest_{n_meshes}_seed{seed}", np.concatenate(Vs), np.concatenate(Fs), voff,
                  foff, np.concatenate(Qs), qoff,
                  meta=dict(meshes=n_meshes, triangles=int(foff[-1]), queries=int(qoff[-1])))


def voxel_grid(V: np.ndarray, res: int = 256, scale: float = 1.05) -> np.ndarray:
    """Voxel-centre grid (res^3 points, x fastest) over the mesh bbox scaled about its centre."""
    lo, hi = V.min(0).astype(np.float64), V.max(0).astype(np.float64)
    c, h = (lo + hi) / 2, (hi - lo) / 2 * scale
    lo2 = c - h
    step = 2 * h / res
    ax = [lo2[a] + (np.arange(res) + 0.5) * step[a] for a in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1).astype(np.float32)


def voxel_workload(nu: int = 500, seeds=(4, 5, 6, 7), res: int = 256) -> Forest:
    Vs, Fs, Qs = [], [], []
    for s in seeds:
        V, F = displaced_icosphere(nu, s)
        Vs.append(V)
        Fs.append(F)
        Qs.append(voxel_grid(V, res))
    voff = np.concatenate([[0], np.cumsum([len(v) for v in Vs])]).astype(np.int64)
    foff = np.concatenate([[0], np.cumsum([len(f) for f in Fs])]).astype(np.int64)
    qoff = np.concatenate([[0], np.cumsum([len(q) for q in Qs])]).astype(np.int64)
    return Forest(f"voxel_{len(seeds)}x_nu{nu}_{res}cubed", np.concatenate(Vs), np.concatenate(Fs),
                  voff, foff, np.concatenate(Qs), qoff,
                  meta=dict(meshes=len(seeds), triangles=int(foff[-1]), queries=int(qoff[-1])))
