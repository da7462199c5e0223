"""CPU oracle for the fast-winding-number path — TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import this
package, and only as the checker / the timed CPU reference; the product path never calls it.

Parity status: UNPINNED against the reference. The reference's arithmetic is in the absent
third-party library jdumas/WindingNumber @ a48b8f555b490afe7aab9159c7daaf83fa2cdf8e
(cmake/recipes/external/winding_number.cmake:21-26) and the reference tests pin no values
(modules/winding/tests/test_fast_winding_number.cpp:80-125). The oracle is pinned by analytic
known-answer tests (tests/test_oracle.py) and committed golden vectors (tests/golden/).

The C sources are in ``fwn_oracle.c`` (O1 FP64 brute force, O2 float Barill tree restating the
reference path, O3 restatement of the device tree builds + FP64 traversal). ``build()`` compiles
them with gcc (``-ffp-contract=off``) into ``oracle/liboracle_fwn.so`` (the checker) and with -O3
into ``oracle/liboracle_fwn_fast.so`` (the timed CPU legs). When a built reference is present
under ``baseline/_ref``, ``ReferenceEngine`` calls the reference's own FastWindingNumber through
``ref_shim.cpp`` (compiled into ``oracle/_ref``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "fwn_oracle.c"
LIB = HERE / "liboracle_fwn.so"
# The same sources built for speed, for the timed CPU legs of the benchmark: -O3 with the
# compiler's default floating-point contraction (the checker build keeps every operation
# separately rounded, which the bit-exact replay of the device build needs; the timed tree
# evaluation O2 does not).
LIB_FAST = HERE / "liboracle_fwn_fast.so"
REF_SHIM = HERE / "ref_shim.cpp"
REF_DIR = HERE.parent / "baseline" / "_ref"
REF_LIB = HERE / "_ref" / "libref_shim.so"

_lib = None
_lib_fast = None
_ref = None


def _compile(out: Path, flags: list[str], force: bool) -> Path:
    if not force and out.exists() and out.stat().st_mtime >= SRC.stat().st_mtime:
        return out
    tmp = out.with_suffix(".so.tmp")
    cmd = ["gcc", *flags, "-std=c11", "-fPIC", "-shared", "-pthread", "-Wall",
           "-Wno-unused-function", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


def build(force: bool = False) -> Path:
    _compile(LIB_FAST, ["-O3", "-funroll-loops"], force)
    return _compile(LIB, ["-O2", "-ffp-contract=off"], force)


def reference_available():
    """(True, path) when a built reference is present under baseline/_ref (its headers and
    liblagrange_winding), with the C shim over its FastWindingNumber compiled into oracle/_ref;
    else (False, why)."""
    inc = REF_DIR / "include" / "lagrange" / "winding" / "FastWindingNumber.h"
    libs = sorted(REF_DIR.glob("**/liblagrange_winding*.so*")) if REF_DIR.exists() else []
    if not inc.exists() or not libs:
        return False, ("no built reference under baseline/_ref (lagrange_winding needs Eigen, "
                       "TBB, spdlog, fmt and jdumas/WindingNumber fetched at configure time; "
                       "the offline install fails)")
    if REF_LIB.exists() and REF_LIB.stat().st_mtime >= REF_SHIM.stat().st_mtime:
        return True, str(REF_LIB)
    REF_LIB.parent.mkdir(exist_ok=True)
    libdirs = sorted({str(p.parent) for p in REF_DIR.glob("**/liblagrange*.so*")})
    cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-pthread", f"-I{REF_DIR / 'include'}",
           str(REF_SHIM), "-o", str(REF_LIB)]
    for d in libdirs:
        cmd += [f"-L{d}", f"-Wl,-rpath,{d}"]
    cmd += ["-llagrange_winding", "-llagrange_core"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return False, "the shim over the reference did not compile: " + r.stderr.strip()[-300:]
    return True, str(REF_LIB)


class ReferenceEngine:
    """The reference's own FastWindingNumber through oracle/ref_shim.cpp (only when
    reference_available() is true)."""

    def __init__(self, V, F):
        global _ref
        ok, path = reference_available()
        if not ok:
            raise RuntimeError(path)
        if _ref is None:
            L = C.CDLL(path)
            L.refshim_build.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64]
            L.refshim_build.restype = C.c_void_p
            L.refshim_free.argtypes = [C.c_void_p]
            L.refshim_query.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                        C.c_void_p, C.c_int]
            _ref = L
        self._V, self._F = _f32(V), _i32(F)
        self.h = _ref.refshim_build(_ptr(self._V), len(self._V), _ptr(self._F), len(self._F))

    def __del__(self):
        if getattr(self, "h", None) and _ref is not None:
            _ref.refshim_free(self.h)
            self.h = None

    def query(self, Q, beta: float = 2.0, nthreads: int | None = None):
        Q = _f32(Q)
        om = np.empty(len(Q), np.float32)
        ins = np.empty(len(Q), np.uint8)
        _ref.refshim_query(self.h, _ptr(Q), len(Q), _ptr(om), _ptr(ins),
                           nthreads or nthreads_default())
        return om, ins


def _bind(L):
    P = C.c_void_p
    i64 = C.c_int64
    L.oracle_ref_build.argtypes = [P, i64, P, i64, C.c_int]
    L.oracle_ref_build.restype = P
    L.oracle_ref_free.argtypes = [P]
    L.oracle_ref_num_nodes.argtypes = [P]
    L.oracle_ref_num_nodes.restype = i64
    L.oracle_ref_query.argtypes = [P, P, i64, C.c_float, P, P, C.c_int]
    L.oracle_ref_query.restype = None
    return L


def lib_fast():
    """The speed build of the same sources (the timed CPU legs only)."""
    global _lib_fast
    if _lib_fast is None:
        build()
        _lib_fast = _bind(C.CDLL(str(LIB_FAST)))
    return _lib_fast


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        i64 = C.c_int64
        L.oracle_brute_f64.argtypes = [P, i64, P, i64, P, i64, P, C.c_int]
        L.oracle_brute_f64.restype = None
        L.oracle_ref_build.argtypes = [P, i64, P, i64, C.c_int]
        L.oracle_ref_build.restype = P
        L.oracle_ref_free.argtypes = [P]
        L.oracle_ref_num_nodes.argtypes = [P]
        L.oracle_ref_num_nodes.restype = i64
        L.oracle_ref_query.argtypes = [P, P, i64, C.c_float, P, P, C.c_int]
        L.oracle_ref_query.restype = None
        L.oracle_lbvh_build.argtypes = [P, P, P, P, i64, C.c_int, C.c_float, C.c_int]
        L.oracle_lbvh_build.restype = P
        L.oracle_lbvh_free.argtypes = [P]
        L.oracle_lbvh_num_nodes.argtypes = [P]
        L.oracle_lbvh_num_nodes.restype = i64
        L.oracle_lbvh_export.argtypes = [P, P, P, P, P, P, P, P, P]
        L.oracle_lbvh_export.restype = None
        L.oracle_lbvh_query_f64.argtypes = [P, P, P, i64, C.c_double, C.c_int, P, C.c_int]
        L.oracle_lbvh_query_f64.restype = None
        L.oracle_tri_solid_angle_f64.argtypes = [P, P, P, P]
        L.oracle_tri_solid_angle_f64.restype = C.c_double
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def nthreads_default() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def tri_solid_angle(v0, v1, v2, q) -> float:
    """Exact FP64 solid angle of one triangle seen from q (Van Oosterom & Strackee 1983)."""
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (v0, v1, v2, q)]
    return lib().oracle_tri_solid_angle_f64(*[_ptr(x) for x in a])


def brute_f64(V, F, Q, nthreads: int | None = None) -> np.ndarray:
    """O1: FP64 solid angle summed over all triangles."""
    V, F, Q = _f32(V), _i32(F), _f32(Q)
    out = np.empty(len(Q), np.float64)
    lib().oracle_brute_f64(_ptr(V), len(V), _ptr(F), len(F), _ptr(Q), len(Q), _ptr(out),
                           nthreads or nthreads_default())
    return out


class RefTree:
    """O2: float order-2 Barill tree, the restatement of the reference FastWindingNumber.
    fast=True uses the speed build (timed CPU legs); the default is the checker build."""

    def __init__(self, V, F, leaf_size: int = 4, fast: bool = False):
        self._L = lib_fast() if fast else lib()
        self._V, self._F = _f32(V), _i32(F)
        self.h = self._L.oracle_ref_build(_ptr(self._V), len(self._V), _ptr(self._F),
                                          len(self._F), leaf_size)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self._L.oracle_ref_free(h)
            self.h = None

    @property
    def num_nodes(self) -> int:
        return self._L.oracle_ref_num_nodes(self.h)

    def query(self, Q, beta: float = 2.0, nthreads: int | None = None):
        Q = _f32(Q)
        om = np.empty(len(Q), np.float32)
        ins = np.empty(len(Q), np.uint8)
        self._L.oracle_ref_query(self.h, _ptr(Q), len(Q), beta, _ptr(om), _ptr(ins),
                                 nthreads or nthreads_default())
        return om, ins


class LbvhTree:
    """O3: CPU restatement of the device tree builds (builder 0: LBVH over Morton codes with a
    Karras hierarchy; builder 1: top-down longest-axis midpoint splits; builder 2: the same with
    binned least-cost planes above 1024 triangles) and of the plain FP64
    traversal."""

    def __init__(self, V, F, leaf_size: int = 8, near_scale: float = 1e-3, voff=None, foff=None,
                 builder: int = 0):
        self._V, self._F = _f32(V), _i32(F)
        if voff is None:
            voff = [0, len(self._V)]
            foff = [0, len(self._F)]
        self.voff = np.ascontiguousarray(voff, dtype=np.int64)
        self.foff = np.ascontiguousarray(foff, dtype=np.int64)
        self.nmeshes = len(self.voff) - 1
        self.h = lib().oracle_lbvh_build(_ptr(self._V), _ptr(self.voff), _ptr(self._F),
                                         _ptr(self.foff), self.nmeshes, leaf_size, near_scale,
                                         builder)
        if not self.h:
            raise ValueError("invalid mesh (index out of range or non-finite vertex)")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().oracle_lbvh_free(h)
            self.h = None

    @property
    def num_nodes(self) -> int:
        return lib().oracle_lbvh_num_nodes(self.h)

    def export(self) -> dict:
        E = self.num_nodes
        nf = int(self.foff[-1])
        out = dict(skip=np.empty(E, np.int32), tri_begin=np.empty(E, np.int32),
                   tri_count=np.empty(E, np.int32), center_radius=np.empty((E, 4), np.float64),
                   moments=np.empty((E, 33), np.float64), sorted_tri=np.empty(nf, np.int32),
                   mesh_root=np.empty((self.nmeshes, 2), np.int32),
                   tau=np.empty(self.nmeshes, np.float32))
        lib().oracle_lbvh_export(self.h, *[_ptr(out[k]) for k in
                                           ("skip", "tri_begin", "tri_count", "center_radius",
                                            "moments", "sorted_tri", "mesh_root", "tau")])
        return out

    def query_f64(self, Q, beta: float = 2.0, exact: bool = False, qmesh=None,
                  nthreads: int | None = None) -> np.ndarray:
        Q = _f32(Q)
        qm = None if qmesh is None else _i32(qmesh)
        out = np.empty(len(Q), np.float64)
        lib().oracle_lbvh_query_f64(self.h, _ptr(Q), _ptr(qm), len(Q), beta, 1 if exact else 0,
                                    _ptr(out), nthreads or nthreads_default())
        return out
