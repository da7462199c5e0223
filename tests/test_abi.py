"""C-ABI surface without a GPU: the library loads, exports every entry point declared in
include/fwn_gb300.h, and rejects invalid arguments before touching the device."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import lagrange_gb300 as fwn

HEADER = Path(__file__).resolve().parent.parent / "include" / "fwn_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"FWN_API\s+[\w\s\*]+?\b(fwn_\w+)\s*\(", text)))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    assert set(fwn.EXPORTS) == set(names), (set(fwn.EXPORTS) ^ set(names))


def test_library_exports_every_declared_symbol(engine_lib):
    for name in declared_functions():
        assert hasattr(engine_lib, name), name
    assert engine_lib.fwn_version().decode().endswith("sm_103a")


def test_config_defaults(engine_lib):
    c = fwn.config_default()
    assert c.beta == 2.0 and c.leaf_size == 8 and c.sort_queries == 1
    assert c.records == fwn.RECORDS_F32 and c.precision == fwn.PRECISION_MIXED
    assert abs(c.fp64_near_scale - 1e-3) < 1e-9


def _build_status(V, nv, F, nf, cfg=None):
    h = C.c_void_p()
    st = fwn.library().fwn_build(V, nv, F, nf, C.byref(cfg) if cfg is not None else None,
                                 C.byref(h))
    buf = C.create_string_buffer(256)
    fwn.library().fwn_last_error(buf, 256)
    return st, buf.value.decode(), h


def test_invalid_arguments_rejected_on_host(engine_lib):
    st, msg, h = _build_status(None, -1, None, 0)
    assert st == 1 and "sizes" in msg and not h.value
    st, msg, _ = _build_status(None, 3, None, 0)
    assert st == 1 and "vertices pointer" in msg
    V = np.zeros((3, 3), np.float32)
    st, msg, _ = _build_status(V.ctypes.data_as(C.c_void_p), 3, None, 1)
    assert st == 1 and "triangles pointer" in msg
    for field, val, frag in (("beta", 0.0, "beta"), ("leaf_size", 17, "leaf_size"),
                             ("leaf_size", 0, "leaf_size"), ("records", 4, "records"),
                             ("block_size", 48, "block_size"), ("precision", 7, "precision"),
                             ("fp64_near_scale", -1.0, "fp64_near_scale"), ("tuning", 8, "tuning"),
                             ("tuning", -1, "tuning"), ("fp64_cond", -1.0, "fp64_cond"),
                             ("builder", 3, "builder")):
        cfg = fwn.config_default(**{field: val})
        st, msg, _ = _build_status(V.ctypes.data_as(C.c_void_p), 3, None, 0, cfg)
        assert st == 1 and frag in msg, (field, msg)


def test_null_handle_is_not_built(engine_lib):
    st = engine_lib.fwn_query_host(None, None, 0, None, None)
    assert st == 6
    assert engine_lib.fwn_query_host_batches(None, 0, None, None, None, None) == 6
    eng = fwn.FastWindingNumber()
    with pytest.raises(fwn.WindingError) as e:
        eng.solid_angle(np.zeros(3, np.float32))
    assert e.value.status == 6


def test_last_error_truncates(engine_lib):
    _build_status(None, -1, None, 0)
    buf = C.create_string_buffer(4)
    n = engine_lib.fwn_last_error(buf, 4)
    assert n > 3 and len(buf.value) == 3


def test_host_mesh_validation():
    with pytest.raises(fwn.WindingError, match="3D"):
        fwn.FastWindingNumber(np.zeros((4, 2), np.float32), np.zeros((1, 3), np.int32))
    with pytest.raises(fwn.WindingError, match="triangle"):
        fwn.FastWindingNumber(np.zeros((4, 3), np.float32), np.zeros((1, 4), np.int32))


def test_forest_sort_key_bits(engine_lib):
    """The forest query's sort-key width comes from the library itself (host-only entry point),
    so the bench's launch count follows the rule the query applies."""
    def offsets(counts):
        return np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)

    assert fwn.forest_sort_key_bits(offsets([10**9])) == 30            # one mesh: Hilbert index
    assert fwn.forest_sort_key_bits(offsets([10**9, 0, 0, 0])) == 32   # 2 mesh bits + 30
    big = [0] * 512
    big[7] = 1 << 20                                                   # 9 mesh bits + 23 bits:
    assert fwn.forest_sort_key_bits(offsets(big)) == 32                # 8 cells per query
    big[7] = (1 << 20) + 1
    assert fwn.forest_sort_key_bits(offsets(big)) == 39                # too coarse: 64-bit keys
    assert fwn.forest_sort_key_bits(offsets([1 << 26, 0, 0, 0, 5])) == 32
    assert fwn.forest_sort_key_bits(offsets([1 << 26, 0, 0, 0, (1 << 26) + 1])) == 33
    L = fwn.library()
    bad = np.array([0, 5, 3], np.int64)
    kb = C.c_int32(0)
    assert L.fwn_forest_sort_key_bits(2, bad.ctypes.data_as(C.c_void_p), C.byref(kb)) == 1
    assert L.fwn_forest_sort_key_bits(0, bad.ctypes.data_as(C.c_void_p), C.byref(kb)) == 1


def test_load_refuses_bad_files_before_device_work(engine_lib, tmp_path):
    """fwn_load checks a file before it touches the device: a missing file, a foreign file and a
    truncated header all return FWN_INVALID_ARG with a message (no GPU is needed to see it)."""
    L = fwn.library()
    h = C.c_void_p()

    def status(path):
        st = L.fwn_load(str(path).encode(), C.byref(h))
        buf = C.create_string_buffer(256)
        L.fwn_last_error(buf, 256)
        return st, buf.value.decode()

    st, msg = status(tmp_path / "missing.fwn")
    assert st == 1 and "cannot open" in msg and not h.value
    (tmp_path / "foreign.fwn").write_bytes(b"NOTANFWN" + bytes(300))
    st, msg = status(tmp_path / "foreign.fwn")
    assert st == 1 and "magic" in msg
    (tmp_path / "short.fwn").write_bytes(b"FWNGB300" + bytes(4))
    st, msg = status(tmp_path / "short.fwn")
    assert st == 1 and "truncated" in msg
    assert L.fwn_load(None, C.byref(h)) == 1
    assert L.fwn_save(None, b"x") == 6


def _engine_file(path, *, skip=1, tri_count=1, root=0, end=1, tri_id=0, flip=False, leaf=8):
    """A one-mesh, one-leaf engine file laid out as fwn_save writes it (header, MeshInfo,
    NodeF32, TriF32, triangle id), with a correct FNV-1a 64 checksum unless `flip`."""
    import struct
    mesh = struct.pack("<2i12f", root, end, *([0.0] * 12))
    node = struct.pack("<4f3if", 0, 0, 0, 1, skip, 0, tri_count, 0) + bytes(96)
    tri = bytes(48)
    payload = bytearray(mesh + node + tri + struct.pack("<i", tri_id))
    h = 1469598103934665603
    for b in payload:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    if flip:
        payload[70] ^= 1
    cfg = bytes(fwn.config_default(leaf_size=8))
    cfg = cfg[:4] + struct.pack("<i", leaf) + cfg[8:]  # leaf_size follows beta
    assert len(cfg) == 64
    header = (b"FWNGB300" + struct.pack("<II", 1, 144) + cfg +
              struct.pack("<5q2i2Q", 3, 1, 1, 1, 1, 1, 0, len(payload), h))
    assert len(header) == 144
    path.write_bytes(header + bytes(payload))
    return path


def test_load_checks_payload_before_device_work(engine_lib, tmp_path):
    """A file whose checksum does not match its payload, or whose node links, triangle ranges,
    mesh roots or triangle ids would send the walk out of bounds, is refused on the host."""
    L = fwn.library()
    h = C.c_void_p()

    def status(path):
        st = L.fwn_load(str(path).encode(), C.byref(h))
        buf = C.create_string_buffer(256)
        L.fwn_last_error(buf, 256)
        return st, buf.value.decode()

    cases = [({"flip": True}, "checksum"), ({"skip": 0}, "inconsistent node"),
             ({"skip": 2}, "inconsistent node"), ({"tri_count": 2}, "inconsistent node"),
             ({"tri_count": 17}, "inconsistent node"), ({"root": 1}, "mesh root"),
             ({"end": 2}, "mesh root"), ({"tri_id": 1}, "triangle id"),
             ({"tri_id": -1}, "triangle id"), ({"leaf": 99}, "leaf_size")]
    for i, (kw, what) in enumerate(cases):
        st, msg = status(_engine_file(tmp_path / f"c{i}.fwn", **kw))
        assert st == 1 and what in msg and not h.value, (kw, msg)



def test_cpp_class_compiles_and_links(engine_lib):
    """The header-only C++ class (the drop-in surface of lagrange::winding::FastWindingNumber)
    compiles with -Wall and links against the library; running it needs a GPU (test_cpp_class)."""
    from lagrange_gb300 import build
    exe = build.build_cpp_test()
    assert exe.exists() and exe.stat().st_size > 0
