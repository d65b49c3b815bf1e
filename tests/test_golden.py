"""Golden fixtures (tests/golden/, written by tests/golden/make_golden.py from the oracle).

CPU: the oracle still reproduces them.  GPU: the library matches them (same tolerances as the
other parity tests)."""
import os

import numpy as np
import pytest

from oracle import mvdecon_oracle as O
from tests.helpers import rel_l2, rel_max

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(HERE, name)))


def decon_inputs(z):
    n = int(z["nviews"])
    return ([z[f"view{i}"] for i in range(n)], [z[f"weight{i}"] for i in range(n)], [z[f"psf{i}"] for i in range(n)])


def test_oracle_reproduces_conv_fixture():
    z = load("conv_12x14x16_k5x3x7.npz")
    np.testing.assert_allclose(O.conv_extended(z["img"], z["kernel"], O.MIRROR), z["mirror"], rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(O.conv_extended(z["img"], z["kernel"], O.VALUE, 1.0), z["value1"], rtol=1e-12,
                               atol=1e-10)


@pytest.mark.parametrize("name", ["decon_cfg1_32x24x16.npz", "decon_cfg2_eb_24x24x20.npz"])
def test_oracle_reproduces_decon_fixture(name):
    z = load(name)
    views, weights, psfs = decon_inputs(z)
    d = O.Deconvolution(views, weights, psfs, int(z["psftype"]), float(z["lam"]), "f64")
    psi = d.run(int(z["iterations"]))
    assert d.avg == pytest.approx(float(z["avg"]), rel=1e-14)
    np.testing.assert_allclose(psi, z["psi"], rtol=1e-10)
    for i in range(len(views)):
        np.testing.assert_allclose(d.k2[i], z[f"k2_{i}"], rtol=1e-10, atol=1e-14)


@pytest.mark.gpu
def test_library_matches_conv_fixture():
    from spim_registration_gb300 import CUDAFourierConvolution

    z = load("conv_12x14x16_k5x3x7.npz")
    out = z["img"].copy()
    CUDAFourierConvolution().convolve3d_inplace(out, list(out.shape), z["kernel"], list(z["kernel"].shape), 0)
    assert rel_max(out, z["mirror"]) < 2e-6


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["decon_cfg1_32x24x16.npz", "decon_cfg2_eb_24x24x20.npz"])
def test_library_matches_decon_fixture(name):
    from spim_registration_gb300 import Deconvolution

    z = load(name)
    views, weights, psfs = decon_inputs(z)
    d = Deconvolution(views, weights, psfs, int(z["psftype"]), float(z["lam"]))
    d.run(int(z["iterations"]))
    assert rel_l2(d.get_psi(), z["psi"]) < 1e-4
    assert d.initial_average() == pytest.approx(float(z["avg"]), rel=1e-12)
    for i in range(len(views)):
        assert rel_max(d.kernel(i, 2), z[f"k2_{i}"]) < 1e-5
