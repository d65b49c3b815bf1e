"""The FP64-free view sum of the weight normalisation (exact_view_sum in
spim_registration_gb300/csrc/inputs.cu), restated on the host in exact_view_sum_check.cpp and
checked against IEEE double sums on random weight sets with zeros, -0, denormals and spread
exponents (no GPU).  The device function itself is compared bit for bit with the oracle in
tests/test_gpu_inputs.py."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_integer_view_sum_matches_double_sums(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "exact_view_sum_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", str(exe), os.path.join(HERE, "exact_view_sum_check.cpp")],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe), "2000000", "11"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    parts = r.stdout.split()
    certified, mismatches = int(parts[3]), int(parts[5])
    assert mismatches == 0
    assert certified > 500000  # the edge-heavy mix still certifies about a third of the sets
