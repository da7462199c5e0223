"""Builds the engine's shared library (CUDA for sm_103a + C++ host code) in-tree.

Output: ``lagrange_gb300/_lib/libfwn_gb300.so`` (C ABI declared in ``include/fwn_gb300.h``),
objects under ``lagrange_gb300/_build/``. Translation units compile in parallel with one
``-gencode`` (sm_103a only). ``lbvh_build.cu`` is compiled with ``-fmad=false`` so that every
floating-point operation of the build is individually rounded in source order (the CPU
restatement of the build reproduces it bit for bit).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libfwn_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
          "-I", str(ROOT / "include")]

# (source, extra flags)
SOURCES = [
    ("radix_sort.cu", []),
    ("lbvh_build.cu", ["-fmad=false"]),
    ("traverse.cu", []),
    ("fwn_capi.cu", []),
    ("noalloc.cu", []),
    ("autotune.cu", []),
    ("callers.cu", []),
    ("probe.cu", []),
    ("persist.cu", []),
]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")
    return exe


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: str, extra: list[str], verbose: bool) -> Path:
    obj = BUILD / (Path(src).stem + ".o")
    deps = [CSRC / src, CSRC / "fwn_internal.cuh", ROOT / "include" / "fwn_gb300.h",
            ROOT / "include" / "lagrange_gb300" / "FastWindingNumber.h"]
    deps = [d for d in deps if d.exists()]
    if not _stale(obj, deps):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    if force:
        for p in BUILD.glob("*.o"):
            p.unlink()
    srcs = [(s, f) for s, f in SOURCES if (CSRC / s).exists()]
    workers = min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(lambda sf: _compile(sf[0], sf[1], verbose), srcs))
    if _stale(LIB, objs) or force:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def build_cpp_test(verbose: bool = False) -> Path:
    """Builds tests/cpp/test_fast_winding_number (C++ class surface test) against the library."""
    src = ROOT / "tests" / "cpp" / "test_fast_winding_number.cpp"
    out = ROOT / "tests" / "cpp" / "_build" / "test_fast_winding_number"
    out.parent.mkdir(parents=True, exist_ok=True)
    deps = [src, LIB, ROOT / "include" / "lagrange_gb300" / "FastWindingNumber.h"]
    if not _stale(out, deps):
        return out
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", str(ROOT / "include"), str(src), "-o", str(out),
           "-L", str(LIBDIR), "-lfwn_gb300", f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for the C++ class test:\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    v = "-v" in sys.argv
    print(build(verbose=v, force="--force" in sys.argv))
