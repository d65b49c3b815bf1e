"""Separable convolution, host side: the oracle against scipy.ndimage's independent 1-D
convolutions, and the Gaussian kernel helpers of CUDASeparableConvolutionFunctions."""
import numpy as np
import pytest

from oracle import mvdecon_oracle as O
from spim_registration_gb300.separable import (SUPPORTED_KERNEL_SIZES, create_gaussian_kernel_1d_double,
                                               get_cuda_kernels, get_float_kernel_padded)


@pytest.mark.parametrize("oob,mode", [(O.SEP_ZERO, "constant"), (O.SEP_VALUE, "constant"), (O.SEP_EXTEND, "nearest")])
def test_oracle_equals_scipy_convolve1d(oob, mode):
    ndimage = pytest.importorskip("scipy.ndimage")
    rng = np.random.default_rng(20)
    img = rng.random((9, 11, 13)).astype(np.float32)
    ks = [rng.standard_normal(7), rng.standard_normal(5), rng.standard_normal(9)]  # asymmetric: orientation
    value = 2.5 if oob == O.SEP_VALUE else 0.0
    got = O.separable_convolve(img, ks, oob, value)
    want = img.astype(np.float64)
    for axis_xyz, k in enumerate(ks):
        want = ndimage.convolve1d(want, k, axis=2 - axis_xyz, mode=mode, cval=value).astype(np.float32).astype(
            np.float64)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-5)


def test_oracle_skips_axes_and_keeps_constants():
    img = np.full((5, 6, 7), 3.0, dtype=np.float32)
    k = create_gaussian_kernel_1d_double(1.5, True)
    out = O.separable_convolve(img, [k, None, k], O.SEP_EXTEND)
    np.testing.assert_allclose(out, 3.0, rtol=1e-6)
    delta = np.zeros(7)
    delta[3] = 1
    rng = np.random.default_rng(2)
    r = rng.random((4, 5, 6)).astype(np.float32)
    np.testing.assert_array_equal(O.separable_convolve(r, [delta, delta, delta], O.SEP_ZERO), r)


def test_gaussian_kernel_rule():
    for sigma in (0.3, 0.5, 1.0, 2.0, 4.7, 10.0):
        k = create_gaussian_kernel_1d_double(sigma, True)
        assert len(k) == max(3, 2 * int(3 * sigma + 0.5) + 1)
        assert k.sum() == pytest.approx(1.0, abs=1e-12)
        np.testing.assert_array_equal(k, k[::-1])
        assert np.argmax(k) == len(k) // 2
    np.testing.assert_array_equal(create_gaussian_kernel_1d_double(0.0, False), [0, 1, 0])


def test_cuda_kernels_are_centred_in_the_smallest_supported_size():
    ks = get_cuda_kernels([1.0, 2.0, 4.0])
    assert {len(k) for k in ks} == {31}  # sigma 4 -> 25 taps -> 31
    g = create_gaussian_kernel_1d_double(1.0, True)
    p = get_float_kernel_padded(g, 31)
    assert p[(31 - len(g)) // 2 + len(g) // 2] == np.float32(g.max())
    assert np.count_nonzero(p) == len(g)
    assert get_cuda_kernels([30.0]) is None  # 181 taps: larger than every supported size
    assert max(SUPPORTED_KERNEL_SIZES) == 127
