"""Integer and float constants the traversal uses in place of conversions and FP64 compares,
read from the CUDA source and checked exhaustively on the CPU."""
import math
import re
from pathlib import Path

import numpy as np

SRC = Path(__file__).resolve().parent.parent / "lagrange_gb300" / "csrc" / "traverse.cu"


def test_inside_threshold_equals_double_compare():
    """inside_of(x) = x > float(0x40C90FDA) must equal (double)x > 2 pi for every float x."""
    text = SRC.read_text()
    m = re.search(r"inside_of\(float res\) \{\s*return res > __int_as_float\((0x[0-9A-Fa-f]+)\)", text)
    assert m, "inside_of not found"
    thr = np.array([int(m.group(1), 16)], np.uint32).view(np.float32)[0]
    bits = np.arange(0x40C80000, 0x40CA0000, dtype=np.uint32)  # every float in [6.25, 6.3125)
    xs = np.concatenate([bits.view(np.float32),
                         np.array([np.nan, np.inf, -np.inf, 0.0, -0.0, 12.566371, -6.2831855],
                                  np.float32)])
    want = xs.astype(np.float64) > 2 * math.pi
    with np.errstate(invalid="ignore"):
        got = xs > thr
    np.testing.assert_array_equal(got, want)


def test_pair_magic_table_divides_exactly():
    """kPairMagic[c] = ceil(2^16 / c), and (p * kPairMagic[c]) >> 16 = p // c for every pair
    index p the leaf loop forms (p < 64 * c, c <= 16)."""
    text = SRC.read_text()
    m = re.search(r"kPairMagic\[WARP_LEAF_MAX \+ 1\] = \{([^}]*)\}", text)
    assert m, "kPairMagic not found"
    table = [int(v.strip().rstrip("u")) for v in m.group(1).split(",")]
    assert len(table) == 17
    for c in range(1, 17):
        assert table[c] == -(-65536 // c)
        p = np.arange(64 * c, dtype=np.uint64)
        np.testing.assert_array_equal((p * table[c]) >> 16, p // c)


def test_key_quantization_matches_truncation():
    """floor by adding 2^23 rounded down (float32) equals int() truncation on [0, 1023]."""
    rng = np.random.default_rng(0)
    u = np.concatenate([rng.uniform(0, 1023, 200_000).astype(np.float32),
                        np.arange(0, 1024, dtype=np.float32),
                        np.nextafter(np.arange(1, 1024, dtype=np.float32), np.float32(0))])
    s = u.astype(np.float64) + 8388608.0        # exact in double
    rd = s.astype(np.float32)                    # nearest; step back where it rounded up
    up = rd.astype(np.float64) > s
    rd[up] = np.nextafter(rd[up], np.float32(0))
    got = rd.view(np.uint32) - np.uint32(0x4B000000)
    np.testing.assert_array_equal(got, u.astype(np.int64).astype(np.uint32))
