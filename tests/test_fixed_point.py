"""The FP32 dJ/dtheta fixed-point conversion that the kernels ship
(sphadjoint_gb300/csrc/sph_fixed.cuh, integer instructions only) gives the
same 128-bit integers as the double-precision form, checked on the host by
compiling the same header with g++."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "sphadjoint_gb300", "csrc")


def test_integer_conversion_equals_double_conversion(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "fixed_point_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC,
                    os.path.join(HERE, "fixed_point_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatches 0" in out.stdout, out.stdout
