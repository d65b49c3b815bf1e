"""The FP64-free arithmetic of the input preparation (spim_registration_gb300/csrc/inputs.cu),
restated on the host and checked against the reference's double arithmetic (no GPU):

* exact_view_sum (exact_view_sum_check.cpp): the sequential double sum of the views' weights
  in 64-bit integers, against IEEE double sums on weight sets with zeros, -0, denormals and
  spread exponents;
* blend_weight (blend_weight_check.cpp): the lookup index Math.round(relDist * 1000.0) from
  FMA sign tests, on quotients beside the half steps, and the certified float-pair product
  against (float)((double)w * lookUp[i]).

The device functions themselves are compared bit for bit with the oracle in
tests/test_gpu_inputs.py."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _run(tmp_path, source, cases, seed):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / os.path.splitext(source)[0]
    # no contraction: the restatements' separate multiplies and adds must stay separate
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", str(exe), os.path.join(HERE, source)],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe), str(cases), str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout.split()


def test_integer_view_sum_matches_double_sums(tmp_path):
    out = _run(tmp_path, "exact_view_sum_check.cpp", 2000000, 11)
    certified, mismatches = int(out[3]), int(out[5])
    assert mismatches == 0
    assert certified > 500000  # the edge-heavy mix still certifies about a third of the sets


def test_blend_index_and_product_match_double_arithmetic(tmp_path):
    out = _run(tmp_path, "blend_weight_check.cpp", 2000000, 5)
    index_mismatches, certified, product_mismatches = int(out[3]), int(out[7]), int(out[9])
    assert index_mismatches == 0 and product_mismatches == 0
    assert certified > 1990000  # the double product decides only near rounding boundaries
