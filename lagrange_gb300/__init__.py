"""GB300 fast-winding-number engine — Python host surface over the C ABI (include/fwn_gb300.h).

Mirrors ``lagrange::winding::FastWindingNumber`` (modules/winding/include/lagrange/winding/
FastWindingNumber.h:24-108): construct from a triangle mesh, then ``solid_angle`` / ``is_inside``
— here over batches of points (numpy arrays on the host, or CUDA tensors already in HBM).

The compiled library ``lagrange_gb300/_lib/libfwn_gb300.so`` is REQUIRED: there is no CPU
fallback. Build it with ``python -c "import __graft_entry__ as g; g.build()"`` (or
``python lagrange_gb300/build.py``).
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

__all__ = ["FastWindingNumber", "Forest", "WindingError", "library", "config_default", "autotune",
           "PRECISION_MIXED", "PRECISION_FP64", "TRAVERSAL_AUTO", "TRAVERSAL_THREAD",
           "TRAVERSAL_WARP", "RECORDS_F32", "RECORDS_F64", "RECORDS_MOMENTS", "BUILDER_LBVH",
           "BUILDER_SPLIT", "BUILDER_BINNED"]

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libfwn_gb300.so"

PRECISION_MIXED, PRECISION_FP64 = 0, 1
TRAVERSAL_AUTO, TRAVERSAL_THREAD, TRAVERSAL_WARP = 0, 1, 2
RECORDS_F32, RECORDS_F64, RECORDS_MOMENTS = 1, 2, 4
BUILDER_LBVH, BUILDER_SPLIT, BUILDER_BINNED = 0, 1, 2

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "TIMEOUT", 5: "INTERNAL",
          6: "NOT_BUILT"}
FOUR_PI = 4.0 * math.pi


class WindingError(RuntimeError):
    """Raised when a C-ABI call returns a non-OK status (the reference raises lagrange::Error)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class fwn_config(C.Structure):
    _fields_ = [("beta", C.c_float), ("leaf_size", C.c_int32), ("records", C.c_int32),
                ("precision", C.c_int32), ("traversal", C.c_int32), ("block_size", C.c_int32),
                ("sort_queries", C.c_int32), ("fp64_near_scale", C.c_float),
                ("fp64_cond", C.c_float), ("tuning", C.c_int32), ("builder", C.c_int32),
                ("reserved", C.c_int32 * 5)]


class fwn_query_opts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("traversal", C.c_int32), ("block_size", C.c_int32),
                ("sort_queries", C.c_int32), ("beta", C.c_float), ("tuning", C.c_int32),
                ("reserved", C.c_int32 * 6)]


class fwn_query_stats(C.Structure):
    _fields_ = [("nodes_tested", C.c_uint64), ("far_evals", C.c_uint64),
                ("tri_evals", C.c_uint64), ("tri_evals_fp64", C.c_uint64),
                ("warp_steps", C.c_uint64)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class fwn_tune_result(C.Structure):
    _fields_ = [("leaf_size", C.c_int32), ("traversal", C.c_int32), ("block_size", C.c_int32),
                ("tuning", C.c_int32), ("ms", C.c_double), ("candidates", C.c_int32),
                ("from_cache", C.c_int32), ("builder", C.c_int32), ("reserved", C.c_int32 * 3)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class fwn_info(C.Structure):
    _fields_ = [("num_vertices", C.c_int64), ("num_triangles", C.c_int64),
                ("num_nodes", C.c_int64), ("num_leaves", C.c_int64), ("num_meshes", C.c_int64),
                ("device_bytes", C.c_int64), ("build_ms", C.c_double),
                ("bbox_min", C.c_float * 3), ("bbox_max", C.c_float * 3),
                ("leaf_size", C.c_int32), ("records", C.c_int32)]


_lib = None

# every entry point declared in include/fwn_gb300.h
EXPORTS = ["fwn_config_default", "fwn_last_error", "fwn_version", "fwn_build", "fwn_build_device",
           "fwn_destroy", "fwn_get_info", "fwn_query", "fwn_query_ex", "fwn_query_host",
           "fwn_query_host_batches", "fwn_export_tree", "fwn_export_moments", "fwn_export_nodes", "fwn_forest_build",
           "fwn_forest_build_device", "fwn_forest_query", "fwn_query_noalloc", "fwn_autotune",
           "fwn_query_grid", "fwn_orientation_criterion", "fwn_query_order",
           "fwn_forest_autotune", "fwn_forest_sort_key_bits", "fwn_probe_fp32_peak",
           "fwn_scratch_pool_stats", "fwn_save", "fwn_load"]


def library():
    """Loads the engine library (raises if it has not been built — no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: the CUDA engine must be built first "
            "(python -c 'import __graft_entry__ as g; g.build()'); there is no CPU fallback")
    L = C.CDLL(str(LIB_PATH))
    P, i64, st = C.c_void_p, C.c_int64, C.c_int
    L.fwn_config_default.argtypes = [C.POINTER(fwn_config)]
    L.fwn_config_default.restype = None
    L.fwn_last_error.argtypes = [C.c_char_p, C.c_size_t]
    L.fwn_last_error.restype = C.c_size_t
    L.fwn_version.argtypes = []
    L.fwn_version.restype = C.c_char_p
    L.fwn_build.argtypes = [P, i64, P, i64, C.POINTER(fwn_config), C.POINTER(P)]
    L.fwn_build_device.argtypes = [P, i64, P, i64, C.POINTER(fwn_config), P, C.POINTER(P)]
    L.fwn_destroy.argtypes = [P]
    L.fwn_get_info.argtypes = [P, C.POINTER(fwn_info)]
    L.fwn_query.argtypes = [P, P, i64, P, P, P]
    L.fwn_query_ex.argtypes = [P, C.POINTER(fwn_query_opts), P, i64, P, P, P,
                               C.POINTER(fwn_query_stats), P]
    L.fwn_query_host.argtypes = [P, P, i64, P, P]
    L.fwn_query_host_batches.argtypes = [P, i64, P, P, P, P]
    L.fwn_query_order.argtypes = [P, P, i64, P, P]
    L.fwn_export_tree.argtypes = [P, P, P, P, P, P, P]
    L.fwn_export_moments.argtypes = [P, P]
    L.fwn_export_nodes.argtypes = [P, P, P]
    L.fwn_forest_build.argtypes = [P, P, P, P, i64, C.POINTER(fwn_config), C.POINTER(P)]
    L.fwn_forest_build_device.argtypes = [P, P, P, P, i64, C.POINTER(fwn_config), P,
                                          C.POINTER(P)]
    L.fwn_forest_query.argtypes = [P, P, P, P, P, C.POINTER(fwn_query_opts), P]
    L.fwn_query_noalloc.argtypes = [P, P, i64, P, P, P]
    L.fwn_query_grid.argtypes = [P, i64, P, P, P, P, P, P]
    L.fwn_orientation_criterion.argtypes = [P, P, i64, P, i64, C.c_float, C.c_float, P, P, P]
    L.fwn_autotune.argtypes = [P, i64, P, i64, P, i64, C.POINTER(fwn_config), C.c_char_p,
                               C.POINTER(fwn_tune_result), P]
    L.fwn_forest_autotune.argtypes = [P, P, P, P, i64, P, P, C.POINTER(fwn_config), C.c_char_p,
                                      C.POINTER(fwn_tune_result), P]
    L.fwn_forest_sort_key_bits.argtypes = [i64, P, C.POINTER(C.c_int32)]
    L.fwn_probe_fp32_peak.argtypes = [C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double), P]
    u64p = C.POINTER(C.c_uint64)
    L.fwn_scratch_pool_stats.argtypes = [C.c_int32, C.c_int32, u64p, u64p, u64p]
    L.fwn_save.argtypes = [P, C.c_char_p]
    L.fwn_load.argtypes = [C.c_char_p, C.POINTER(P)]
    for name in ("fwn_build", "fwn_build_device", "fwn_destroy", "fwn_get_info", "fwn_query",
                 "fwn_query_ex", "fwn_query_host", "fwn_query_host_batches", "fwn_export_tree",
                 "fwn_export_moments", "fwn_export_nodes",
                 "fwn_forest_build", "fwn_forest_build_device", "fwn_forest_query",
                 "fwn_query_noalloc", "fwn_autotune", "fwn_query_grid",
                 "fwn_orientation_criterion", "fwn_query_order", "fwn_forest_autotune",
                 "fwn_forest_sort_key_bits", "fwn_probe_fp32_peak", "fwn_scratch_pool_stats",
                 "fwn_save", "fwn_load"):
        getattr(L, name).restype = st
    _lib = L
    return L


def _check(status: int):
    if status != 0:
        buf = C.create_string_buffer(1024)
        library().fwn_last_error(buf, 1024)
        raise WindingError(status, buf.value.decode(errors="replace"))


def config_default(**overrides) -> fwn_config:
    c = fwn_config()
    library().fwn_config_default(C.byref(c))
    for k, v in overrides.items():
        if not hasattr(c, k):
            raise TypeError(f"unknown config field {k!r}")
        setattr(c, k, v)
    return c


def forest_sort_key_bits(query_offsets) -> int:
    """Key width (bits) of the radix sort fwn_forest_query runs for these query offsets
    [num_meshes + 1]; the sort makes ceil(bits / 8) passes. Host-only."""
    q = np.ascontiguousarray(np.asarray(query_offsets), dtype=np.int64)
    out = C.c_int32(0)
    _check(library().fwn_forest_sort_key_bits(len(q) - 1, q.ctypes.data_as(C.c_void_p),
                                              C.byref(out)))
    return int(out.value)


def scratch_pool_stats(device: int = 0, reset_high: bool = False) -> dict:
    """Bytes the library's query-scratch pool of `device` reserves, hands out, and has handed out
    at most since the last reset (fwn_scratch_pool_stats)."""
    r, u, h = C.c_uint64(0), C.c_uint64(0), C.c_uint64(0)
    _check(library().fwn_scratch_pool_stats(int(device), 1 if reset_high else 0, C.byref(r),
                                            C.byref(u), C.byref(h)))
    return {"reserved": r.value, "used": u.value, "used_high": h.value}


def probe_fp32_peak(form: int = 0, stream=None) -> dict:
    """Measured FP32 FMA throughput of the current device (fwn_probe_fp32_peak): form 0 scalar
    FMA, 1 paired f32x2 FMA. Returns {"tflops", "flops", "ms"}."""
    fl, ms = C.c_double(0.0), C.c_double(0.0)
    _check(library().fwn_probe_fp32_peak(int(form), C.byref(fl), C.byref(ms), _stream_ptr(stream)))
    return {"tflops": fl.value / (ms.value * 1e-3) / 1e12, "flops": fl.value, "ms": ms.value}


def _opts(precision=None, traversal=None, block_size=None, sort_queries=None, beta=None,
          tuning=None):
    o = fwn_query_opts()
    o.precision = -1 if precision is None else int(precision)
    o.traversal = -1 if traversal is None else int(traversal)
    o.block_size = 0 if block_size is None else int(block_size)
    o.sort_queries = -1 if sort_queries is None else int(sort_queries)
    o.beta = 0.0 if beta is None else float(beta)
    o.tuning = 0 if tuning is None else int(tuning)
    return o


def _is_cuda_tensor(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


def _stream_ptr(stream):
    if stream is None:
        try:
            import torch
            return C.c_void_p(torch.cuda.current_stream().cuda_stream)
        except Exception:
            return C.c_void_p(0)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


def _host_mesh(vertices, facets):
    V = np.ascontiguousarray(np.asarray(vertices), dtype=np.float32)   # FastWindingNumber.cpp:40-44
    F = np.ascontiguousarray(np.asarray(facets), dtype=np.int64)
    if V.ndim != 2 or V.shape[1] != 3:
        raise WindingError(1, "Fast winding number engine only supports 3D meshes")
    if F.size and (F.ndim != 2 or F.shape[1] != 3):
        raise WindingError(1, "Fast winding number engine only supports triangle meshes")
    F = F.reshape(-1, 3)
    # indices are cast to int (FastWindingNumber.cpp:46-50); out-of-range ones are rejected by
    # the device build
    F32 = F.astype(np.int32)
    if F.size and (F.max() > np.iinfo(np.int32).max or F.min() < np.iinfo(np.int32).min):
        raise WindingError(1, "triangle vertex index out of range")
    return V, F32


class FastWindingNumber:
    """Winding-number engine for one triangle mesh.

    ``FastWindingNumber(vertices [nv,3], facets [nf,3], beta=2, leaf_size=8, ...)``.
    Host numpy inputs use the synchronous host path; CUDA tensors stay on the device. The engine
    lives on the device it was built on (the tensors' device, or the current device for host
    inputs); CUDA-tensor calls run with the tensors' device made current, and the library rejects
    a call whose device is not the engine's.
    """

    def __init__(self, vertices=None, facets=None, *, config: fwn_config | None = None,
                 **cfg_overrides):
        self._h = C.c_void_p(None)
        if vertices is None:
            return  # default-constructed: queries raise NOT_BUILT
        cfg = config if config is not None else config_default(**cfg_overrides)
        L = library()
        if _is_cuda_tensor(vertices):
            import torch
            V = vertices.detach().to(torch.float32).contiguous()
            F = facets.detach().to(torch.int32).contiguous()
            if V.dim() != 2 or V.shape[1] != 3:
                raise WindingError(1, "Fast winding number engine only supports 3D meshes")
            with torch.cuda.device(V.device):
                _check(L.fwn_build_device(C.c_void_p(V.data_ptr()), V.shape[0],
                                          C.c_void_p(F.data_ptr()), F.shape[0] if F.numel() else 0,
                                          C.byref(cfg), _stream_ptr(None), C.byref(self._h)))
        else:
            V, F = _host_mesh(vertices, facets)
            _check(L.fwn_build(V.ctypes.data_as(C.c_void_p), len(V),
                               F.ctypes.data_as(C.c_void_p), len(F), C.byref(cfg),
                               C.byref(self._h)))

    def save(self, path) -> None:
        """Writes the built engine to a file (fwn_save); `load` reads it back without a build."""
        _check(library().fwn_save(self._h, str(path).encode()))

    @classmethod
    def load(cls, path):
        """An engine read from a file written by `save`, on the current device (fwn_load)."""
        obj = cls.__new__(cls)
        obj._h = C.c_void_p(None)
        _check(library().fwn_load(str(path).encode(), C.byref(obj._h)))
        return obj

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            library().fwn_destroy(self._h)
            self._h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def info(self) -> dict:
        i = fwn_info()
        _check(library().fwn_get_info(self._h, C.byref(i)))
        d = {k: getattr(i, k) for k, _ in fwn_info._fields_}
        d["bbox_min"] = list(i.bbox_min)
        d["bbox_max"] = list(i.bbox_max)
        return d

    # ---- queries -------------------------------------------------------------------------
    def query(self, points, *, omega=True, inside=True, precision=None, traversal=None,
              block_size=None, sort_queries=None, beta=None, omega_f64=False, stats=False,
              stream=None):
        """Returns (omega, inside[, omega_f64][, stats]) for a batch of points.

        numpy input -> numpy outputs (host path, synchronous unless options are given, in which
        case a device round trip through torch is used). CUDA tensor input -> CUDA tensors.
        """
        L = library()
        o = _opts(precision, traversal, block_size, sort_queries, beta)
        if _is_cuda_tensor(points):
            import torch
            Q = points.detach().to(torch.float32).contiguous().reshape(-1, 3)
            n = Q.shape[0]
            dev = Q.device
            w = torch.empty(n, dtype=torch.float32, device=dev) if omega else None
            ins = torch.empty(n, dtype=torch.uint8, device=dev) if inside else None
            w64 = torch.empty(n, dtype=torch.float64, device=dev) if omega_f64 else None
            st = fwn_query_stats() if stats else None
            ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
            with torch.cuda.device(dev):
                _check(L.fwn_query_ex(self._h, C.byref(o), ptr(Q), n, ptr(w), ptr(ins), ptr(w64),
                                      C.byref(st) if st is not None else None, _stream_ptr(stream)))
            out = (w, ins)
            if omega_f64:
                out = out + (w64,)
            if stats:
                out = out + (st.as_dict(),)
            return out
        Q = np.ascontiguousarray(np.asarray(points), dtype=np.float32).reshape(-1, 3)
        plain = all(v is None for v in (precision, traversal, block_size, sort_queries, beta)) \
            and not omega_f64 and not stats
        if plain:
            n = len(Q)
            w = np.empty(n, np.float32) if omega else None
            ins = np.empty(n, np.uint8) if inside else None
            pw = w.ctypes.data_as(C.c_void_p) if w is not None else None
            pi = ins.ctypes.data_as(C.c_void_p) if ins is not None else None
            _check(L.fwn_query_host(self._h, Q.ctypes.data_as(C.c_void_p), n, pw, pi))
            return w, ins
        import torch
        res = self.query(torch.from_numpy(Q).cuda(), omega=omega, inside=inside,
                         precision=precision, traversal=traversal, block_size=block_size,
                         sort_queries=sort_queries, beta=beta, omega_f64=omega_f64, stats=stats,
                         stream=stream)
        torch.cuda.synchronize()
        return tuple(r.cpu().numpy() if hasattr(r, "cpu") else r for r in res)

    def query_host_batches(self, batches, omega=True, inside=True):
        """Queries a list of host point sets ([n_b, 3] float32 numpy arrays or CPU tensors) in
        one call (fwn_query_host_batches): batch b's copy in and batch b - 1's copy out overlap
        the walk of the batch between them. Returns a list of (omega, inside) per batch, each
        as fwn_query_host returns it, in the input's kind (numpy, or CPU tensors; pinned when
        the input is pinned, which the copies need to overlap)."""
        L = library()
        nb = len(batches)
        ins_, outs = [], []
        for b in batches:
            if hasattr(b, "is_pinned"):
                import torch
                Q = b.detach().to(torch.float32).contiguous().reshape(-1, 3)
                if Q.is_cuda:
                    raise ValueError("query_host_batches takes host point sets")
                pin = Q.is_pinned()
                mk = (lambda n, dt: torch.empty(n, dtype=dt).pin_memory()) if pin else \
                    (lambda n, dt: torch.empty(n, dtype=dt))
                w = mk(Q.shape[0], torch.float32) if omega else None
                i = mk(Q.shape[0], torch.uint8) if inside else None
                ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
            else:
                Q = np.ascontiguousarray(np.asarray(b), dtype=np.float32).reshape(-1, 3)
                w = np.empty(len(Q), np.float32) if omega else None
                i = np.empty(len(Q), np.uint8) if inside else None
                ptr = lambda t: t.ctypes.data if t is not None else None  # noqa: E731
            ins_.append(Q)
            outs.append((w, i, ptr(Q), ptr(w), ptr(i)))
        pts = (C.c_void_p * max(nb, 1))(*[o[2] for o in outs])
        cnt = (C.c_int64 * max(nb, 1))(*[int(q.shape[0]) for q in ins_])
        pw = (C.c_void_p * max(nb, 1))(*[o[3] for o in outs]) if omega else None
        pi = (C.c_void_p * max(nb, 1))(*[o[4] for o in outs]) if inside else None
        _check(L.fwn_query_host_batches(self._h, nb, pts, cnt, pw, pi))
        return [(o[0], o[1]) for o in outs]

    def query_order(self, points, stream=None):
        """The permutation the query applies to group nearby points into warps (int64 CUDA
        tensor): points[order] queried with sort_queries=False gives the same results."""
        import torch
        Q = points.detach().to(torch.float32).contiguous().reshape(-1, 3)
        n = Q.shape[0]
        o = torch.empty(n, dtype=torch.int32, device=Q.device)  # uint32 bits, n < 2^31
        with torch.cuda.device(Q.device):
            _check(library().fwn_query_order(self._h, C.c_void_p(Q.data_ptr()), n,
                                             C.c_void_p(o.data_ptr()), _stream_ptr(stream)))
        return o.long()

    def solid_angle(self, points):
        """Solid angle(s) in steradians (FastWindingNumber.cpp:69-76). A single point (3,)
        returns a float, a batch (n,3) an array."""
        single = np.ndim(points) == 1 and not _is_cuda_tensor(points)
        w, _ = self.query(points, inside=False)
        return float(w[0]) if single else w

    def is_inside(self, points):
        """Omega/(4 pi) > 0.5 (FastWindingNumber.cpp:60-67)."""
        single = np.ndim(points) == 1 and not _is_cuda_tensor(points)
        _, ins = self.query(points, omega=False)
        return bool(ins[0]) if single else (ins.astype(bool) if isinstance(ins, np.ndarray) else ins)

    # ---- callers of the path ----------------------------------------------------------------
    def query_grid(self, origin, spacing, dims, *, mesh: int = 0, omega=True, inside=True,
                   stream=None):
        """Voxel-grid sign pass: classifies the centres of a dims = (nx, ny, nz) grid, centre of
        voxel (i, j, k) = origin + (i + 0.5, j + 0.5, k + 0.5) * spacing (one fused rounding per
        axis). Returns CUDA tensors of shape (nz, ny, nx) (x fastest)."""
        import torch
        nx, ny, nz = (int(d) for d in dims)
        o = (C.c_float * 3)(*[float(x) for x in origin])
        s = (C.c_float * 3)(*[float(x) for x in spacing])
        d = (C.c_int64 * 3)(nx, ny, nz)
        n = nx * ny * nz
        w = torch.empty(n, dtype=torch.float32, device="cuda") if omega else None
        ins = torch.empty(n, dtype=torch.uint8, device="cuda") if inside else None
        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        _check(library().fwn_query_grid(self._h, mesh, o, s, d, ptr(w), ptr(ins),
                                        _stream_ptr(stream)))
        shape = (nz, ny, nx)
        return (w.view(shape) if w is not None else None,
                ins.view(shape) if ins is not None else None)

    def orientation_criterion(self, vertices, facets, *, eps: float = 1e-2,
                              threshold: float = 0.8, stream=None):
        """Per-facet orientation test of another mesh against this (reference) mesh:
        criterion = (Omega(b + eps n) - Omega(b - eps n)) / (4 pi), flip = criterion > threshold
        (modules/winding/examples/fix_orientation.cpp:75-115). Returns CUDA tensors."""
        import torch
        V = vertices if _is_cuda_tensor(vertices) else torch.from_numpy(
            np.ascontiguousarray(vertices, np.float32)).cuda()
        F = facets if _is_cuda_tensor(facets) else torch.from_numpy(
            np.ascontiguousarray(facets, np.int32)).cuda()
        V = V.to(torch.float32).contiguous()
        F = F.to(torch.int32).contiguous().reshape(-1, 3)
        nf = F.shape[0]
        crit = torch.empty(nf, dtype=torch.float32, device=V.device)
        flip = torch.empty(nf, dtype=torch.uint8, device=V.device)
        with torch.cuda.device(V.device):
            _check(library().fwn_orientation_criterion(
                self._h, C.c_void_p(V.data_ptr()), V.shape[0], C.c_void_p(F.data_ptr()), nf,
                float(eps), float(threshold), C.c_void_p(crit.data_ptr()),
                C.c_void_p(flip.data_ptr()), _stream_ptr(stream)))
        return crit, flip

    def sample_inside(self, num_samples: int, *, seed: int = 0):
        """Rejection sampling of interior points (modules/winding/examples/
        sample_points_in_mesh.cpp:59-76): num_samples uniform points in the mesh bbox, kept where
        is_inside holds. Returns a CUDA tensor (k, 3)."""
        import torch
        inf = self.info()
        lo = torch.tensor(inf["bbox_min"], dtype=torch.float32, device="cuda")
        hi = torch.tensor(inf["bbox_max"], dtype=torch.float32, device="cuda")
        g = torch.Generator(device="cuda").manual_seed(seed)
        P = lo + (hi - lo) * torch.rand((int(num_samples), 3), generator=g, device="cuda")
        _, ins = self.query(P, omega=False)
        return P[ins.bool()]

    # ---- inspection ------------------------------------------------------------------------
    def export_tree(self) -> dict:
        inf = self.info()
        E, nf, M = inf["num_nodes"], inf["num_triangles"], inf["num_meshes"]
        out = dict(skip=np.empty(E, np.int32), tri_begin=np.empty(E, np.int32),
                   tri_count=np.empty(E, np.int32), center_radius=np.empty((E, 4), np.float64),
                   sorted_tri=np.empty(nf, np.int32), mesh_root=np.empty((M, 2), np.int32))
        p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        _check(library().fwn_export_tree(self._h, p(out["skip"]), p(out["tri_begin"]),
                                         p(out["tri_count"]), p(out["center_radius"]),
                                         p(out["sorted_tri"]), p(out["mesh_root"])))
        return out

    def export_nodes(self) -> dict:
        """The device node records as arrays: "f32" [E, 32] float32 and "f64" [E, 32] float64
        (the raw 128 B / 256 B records; the integer fields read as their bit patterns), each
        present when the engine keeps that record set."""
        inf = self.info()
        E = inf["num_nodes"]
        out = {}
        rec = inf.get("records", RECORDS_F32)
        n32 = np.zeros((E, 32), np.float32) if rec & RECORDS_F32 else None
        n64 = np.zeros((E, 32), np.float64) if rec & RECORDS_F64 else None
        p = lambda a: a.ctypes.data_as(C.c_void_p) if a is not None else None  # noqa: E731
        _check(library().fwn_export_nodes(self._h, p(n32), p(n64)))
        if n32 is not None:
            out["f32"] = n32
        if n64 is not None:
            out["f64"] = n64
        return out

    def export_moments(self) -> np.ndarray:
        E = self.info()["num_nodes"]
        m = np.empty((E, 33), np.float64)
        _check(library().fwn_export_moments(self._h, m.ctypes.data_as(C.c_void_p)))
        return m


class Forest(FastWindingNumber):
    """Many meshes built and queried together (one launch per stage over all meshes)."""

    def __init__(self, vertices, voff, facets, foff, *, config: fwn_config | None = None,
                 **cfg_overrides):
        self._h = C.c_void_p(None)
        cfg = config if config is not None else config_default(**cfg_overrides)
        self.voff = np.ascontiguousarray(voff, dtype=np.int64)
        self.foff = np.ascontiguousarray(foff, dtype=np.int64)
        self.nmeshes = len(self.voff) - 1
        L = library()
        if _is_cuda_tensor(vertices):
            import torch
            V = vertices.detach().to(torch.float32).contiguous()
            F = facets.detach().to(torch.int32).contiguous()
            with torch.cuda.device(V.device):
                _check(L.fwn_forest_build_device(C.c_void_p(V.data_ptr()),
                                                 self.voff.ctypes.data_as(C.c_void_p),
                                                 C.c_void_p(F.data_ptr()),
                                                 self.foff.ctypes.data_as(C.c_void_p), self.nmeshes,
                                                 C.byref(cfg), _stream_ptr(None), C.byref(self._h)))
        else:
            V = np.ascontiguousarray(vertices, dtype=np.float32)
            F = np.ascontiguousarray(facets, dtype=np.int32)
            _check(L.fwn_forest_build(V.ctypes.data_as(C.c_void_p),
                                      self.voff.ctypes.data_as(C.c_void_p),
                                      F.ctypes.data_as(C.c_void_p),
                                      self.foff.ctypes.data_as(C.c_void_p), self.nmeshes,
                                      C.byref(cfg), C.byref(self._h)))

    def query_forest(self, points, qoff, *, precision=None, traversal=None, block_size=None,
                     sort_queries=None, beta=None, stream=None):
        """points: CUDA tensor [sum Q, 3]; qoff: host int64 offsets [M+1]."""
        import torch
        qoff = np.ascontiguousarray(qoff, dtype=np.int64)
        Q = points.detach().to(torch.float32).contiguous().reshape(-1, 3)
        n = Q.shape[0]
        w = torch.empty(n, dtype=torch.float32, device=Q.device)
        ins = torch.empty(n, dtype=torch.uint8, device=Q.device)
        o = _opts(precision, traversal, block_size, sort_queries, beta)
        with torch.cuda.device(Q.device):
            _check(library().fwn_forest_query(self._h, C.c_void_p(Q.data_ptr()),
                                              qoff.ctypes.data_as(C.c_void_p),
                                              C.c_void_p(w.data_ptr()), C.c_void_p(ins.data_ptr()),
                                              C.byref(o), _stream_ptr(stream)))
        return w, ins


def autotune(vertices, facets, points, *, cache_path=None, config: fwn_config | None = None,
             **cfg_overrides) -> dict:
    """Times every (leaf size, schedule, block, variant) candidate on a sample of query points
    and returns the fastest; ``result["config"]`` can be passed as keyword arguments to
    ``FastWindingNumber``. With ``cache_path`` the choice is cached per GPU and size bucket."""
    import torch
    V = torch.as_tensor(np.asarray(vertices, np.float32)).cuda() if not _is_cuda_tensor(vertices) \
        else vertices.detach().to(torch.float32).contiguous()
    F = torch.as_tensor(np.asarray(facets, np.int32)).cuda() if not _is_cuda_tensor(facets) \
        else facets.detach().to(torch.int32).contiguous()
    Q = torch.as_tensor(np.asarray(points, np.float32)).cuda() if not _is_cuda_tensor(points) \
        else points.detach().to(torch.float32).contiguous()
    cfg = config if config is not None else config_default(**cfg_overrides)
    r = fwn_tune_result()
    _check(library().fwn_autotune(C.c_void_p(V.data_ptr()), V.shape[0], C.c_void_p(F.data_ptr()),
                                  F.shape[0], C.c_void_p(Q.data_ptr()), Q.reshape(-1, 3).shape[0],
                                  C.byref(cfg), cache_path.encode() if cache_path else None,
                                  C.byref(r), _stream_ptr(None)))
    d = r.as_dict()
    d["config"] = {"leaf_size": r.leaf_size, "traversal": r.traversal,
                   "block_size": r.block_size, "tuning": r.tuning, "builder": r.builder}
    return d


def autotune_forest(vertices, voff, facets, foff, points, qoff, *, cache_path=None,
                    config: fwn_config | None = None, **cfg_overrides) -> dict:
    """Picks the builder, leaf size and register-cap variant of a forest by building it for
    every candidate builder and leaf size and timing the persistent forest query on ``points`` (CUDA tensor or array, [sum Q, 3]) with host offsets
    ``qoff``; ``result["config"]`` can be passed to ``Forest``."""
    import torch

    def dev(x, dt):
        return x.detach().to(dt).contiguous() if _is_cuda_tensor(x) else \
            torch.as_tensor(np.asarray(x)).to(dt).cuda().contiguous()
    V, F, Q = dev(vertices, torch.float32), dev(facets, torch.int32), dev(points, torch.float32)
    vo, fo, qo = (np.ascontiguousarray(o, dtype=np.int64) for o in (voff, foff, qoff))
    cfg = config if config is not None else config_default(**cfg_overrides)
    r = fwn_tune_result()
    _check(library().fwn_forest_autotune(
        C.c_void_p(V.data_ptr()), vo.ctypes.data_as(C.c_void_p), C.c_void_p(F.data_ptr()),
        fo.ctypes.data_as(C.c_void_p), len(vo) - 1, C.c_void_p(Q.data_ptr()),
        qo.ctypes.data_as(C.c_void_p), C.byref(cfg), cache_path.encode() if cache_path else None,
        C.byref(r), _stream_ptr(None)))
    d = r.as_dict()
    d["config"] = {"leaf_size": r.leaf_size, "tuning": r.tuning, "builder": r.builder}
    return d

