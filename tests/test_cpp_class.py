"""Runs the C++ class-surface test (tests/cpp/test_fast_winding_number.cpp) on the GPU."""
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_cpp_class_surface(engine_lib):
    from lagrange_gb300 import build
    exe = build.build_cpp_test()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK" in r.stdout
