"""The integer FP64 product used by the push kernels equals the native double multiply
bit for bit (host build of the same header the kernels include)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c2g_mul_matches_native_double(tmp_path):
    exe = str(tmp_path / "fp64_mul_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "c-2graph_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "fp64_mul_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, "3000000"], check=True, capture_output=True, text=True).stdout
    assert out.startswith("ok "), out
    assert int(out.split()[1]) > 3000000
