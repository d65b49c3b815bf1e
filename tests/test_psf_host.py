"""PSF pipeline, host side: the oracle's ExtractPSF restatement on known answers, and the
library's host-only transformed-size entry against it."""
import math

import numpy as np
import pytest

from oracle import mvdecon_oracle as O
from spim_registration_gb300 import native
from spim_registration_gb300.psf import make_same_size


def _rot_y(deg, scale=(1.0, 1.0, 1.0), shift=(0.0, 0.0, 0.0)):
    t = math.radians(deg)
    r = np.array([[math.cos(t), 0, math.sin(t)], [0, 1, 0], [-math.sin(t), 0, math.cos(t)]]) @ np.diag(scale)
    return np.concatenate([r, np.asarray(shift, dtype=np.float64)[:, None]], axis=1).ravel()


def test_single_integer_location_extracts_the_neighbourhood_periodically():
    rng = np.random.default_rng(1)
    img = rng.random((10, 12, 14))
    psf = O.extract_psf_local(img, [(1, 6, 5)], (5, 3, 7))  # x = 1: the box wraps around in x
    z, y, x = np.meshgrid(np.arange(7) - 3 + 5, np.arange(3) - 1 + 6, np.arange(5) - 2 + 1, indexing="ij")
    np.testing.assert_allclose(psf, img[z % 10, y % 12, x % 14], rtol=1e-12)


def test_locations_add_and_normalise_to_unit_range():
    rng = np.random.default_rng(2)
    img = rng.random((16, 16, 16))
    a = O.extract_psf_local(img, [(4.25, 5.5, 6.75)], (5, 5, 5))
    b = O.extract_psf_local(img, [(9.0, 3.0, 11.5)], (5, 5, 5))
    ab = O.extract_psf_local(img, [(4.25, 5.5, 6.75), (9.0, 3.0, 11.5)], (5, 5, 5))
    np.testing.assert_allclose(ab, a + b, rtol=1e-12)
    n = O.extract_psf_local(img, [(4.25, 5.5, 6.75)], (5, 5, 5), normalize=True)
    assert n.min() == 0 and n.max() == pytest.approx(1.0)


def test_transformed_size_identity_and_rotation():
    dims, off = O.transformed_psf_size((9, 11, 21), _rot_y(0))
    assert dims == [9, 11, 21] and np.allclose(off, 0)
    dims, off = O.transformed_psf_size((9, 11, 21), _rot_y(90))
    assert dims == [21, 11, 9]
    psf = np.random.default_rng(3).random((21, 11, 9))
    out = O.transform_psf(psf, _rot_y(0), (9, 11, 21), (0, 0, 0))
    np.testing.assert_allclose(out, psf, atol=1e-12)
    dims, off = O.transformed_psf_size((8, 11, 21), _rot_y(0))
    assert dims[0] == 9  # even extent + 1 is made odd


@pytest.mark.parametrize("deg,scale", [(0, (1, 1, 1)), (30, (1, 1, 2.5)), (90, (1, 1, 1.7)), (137, (1.2, 0.9, 2))])
def test_library_transformed_size_matches_the_oracle(deg, scale):
    lib = native.load()
    m = _rot_y(deg, scale, (3.0, -2.0, 7.5))
    dims = (native.ctypes.c_int * 3)()
    off = (native.ctypes.c_double * 3)()
    native.check(lib.mvd_transformed_psf_size(native.iarr([11, 13, 25]), (native.ctypes.c_double * 12)(*m), dims,
                                              off))
    want_dims, want_off = O.transformed_psf_size((11, 13, 25), m)
    assert list(dims) == want_dims
    np.testing.assert_allclose(list(off), want_off, rtol=1e-12, atol=1e-12)
    assert all(d % 2 == 1 for d in dims)


def test_make_same_size_centres_and_fills_with_the_minimum():
    img = np.arange(27, dtype=np.float32).reshape(3, 3, 3) + 5
    out = make_same_size(img, (7, 5, 9))
    assert out.shape == (9, 5, 7)
    np.testing.assert_array_equal(out[3:6, 1:4, 2:5], img)
    assert out[0, 0, 0] == 5
