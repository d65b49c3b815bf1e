"""Precision of the FP32 GPU path against the FP64 oracle (the method's precision config).

Configuration 4's PSF (31x31x61, sigma 2,2,7) and four rotated views on a reduced volume
(96x96x64) that the FP64 oracle runs in seconds.  Every output volume -- psi after 10 and
after 50 iterations -- has its relative L2 and max-abs error against FP64 stated (printed) and
bounded: relative L2 <= 1e-4 after 10 iterations (the method's gate) and after 50.
"""
import numpy as np
import pytest

from oracle import mvdecon_oracle as O
from spim_registration_gb300 import Deconvolution
from spim_registration_gb300 import synthetic as S
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


def test_cfg4_shapes_fp32_against_fp64():
    p = S.make_problem(4, shape_xyz=(96, 96, 64), n_blobs=60, iterations=50)
    d = Deconvolution(p.views, p.weights, p.psfs, p.psftype, p.lam)
    o = O.Deconvolution(p.views, p.weights, p.psfs, p.psftype, p.lam, "f64")
    report = {}
    done = 0
    for stop in (10, 50):
        d.run(stop - done)
        o.run(stop - done)
        done = stop
        got, ref = d.get_psi().astype(np.float64), o.psi
        report[stop] = (rel_l2(got, ref), float(np.abs(got - ref).max()), float(np.abs(ref).max()))
    for it, (rl2, mx, scale) in report.items():
        print(f"cfg4 shapes, {it} iterations: relative L2 {rl2:.3e}, max abs {mx:.3e} (max |psi| {scale:.3e})")
    assert report[10][0] <= 1e-4
    assert report[50][0] <= 1e-4
