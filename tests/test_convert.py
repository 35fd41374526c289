"""The integer-pipe double <-> float conversions of the update and mirror
kernels (spheral_gb300/csrc/convert.cuh) give the bits of the IEEE
round-to-nearest-even casts: random bit patterns, values across the float
range, ties at every exponent and the special values, checked by a small C++
program built with g++ against the host's casts (the device falls back to
the conversion instruction exactly where the host code does)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_conversions_match_ieee_casts(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "convert_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "spheral_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "convert_check.cc"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
