"""Parity of the drop-in convolve-in-place C ABI against the CPU oracle (GPU).

The calls go through ctypes exactly as JNA issues them from MVDeconFFTThreads
(float32 x-fastest block, dims reversed {z, y, x}).  Tolerance: FP32 FFT convolution vs the
FP64 oracle, max abs error <= 2e-6 of the output's max (relative L2 reported too).
"""
import numpy as np
import pytest

from oracle import mvdecon_oracle as O
from spim_registration_gb300 import CUDAFourierConvolution, synthetic as S
from spim_registration_gb300.native import MvdError
from tests.helpers import rel_l2, rel_max

pytestmark = pytest.mark.gpu

TOL = 2e-6


@pytest.fixture(scope="module")
def cuda():
    c = CUDAFourierConvolution()
    assert c.getNumDevicesCUDA() >= 1
    return c


def conv_case(cuda, shape_zyx, kshape_zyx, seed=0):
    r = np.random.default_rng(seed)
    im = (r.random(shape_zyx) * 100).astype(np.float32)
    k = r.random(kshape_zyx).astype(np.float32)
    k /= k.sum()
    ref = O.conv_extended(im, k, O.MIRROR, 0.0, "f64")
    out = im.copy()
    cuda.convolution3DfftCUDAInPlace(out, list(shape_zyx), k, list(kshape_zyx), 0)
    assert cuda.last_error() == ""
    return out, ref


@pytest.mark.parametrize(
    "shape,kshape",
    [
        ((16, 16, 16), (9, 5, 5)),
        ((11, 13, 17), (7, 5, 3)),          # odd / prime sizes
        ((40, 48, 64), (25, 9, 9)),
        ((1, 8, 9), (1, 3, 5)),             # single slice, mirror-single of a length-1 axis
        ((6, 5, 9), (11, 7, 3)),            # kernel larger than the block along z and y
        ((88, 136, 136), (25, 9, 9)),       # the single block of 128x128x64 with a 9x9x25 PSF
        ((128, 128, 128), (41, 15, 15)),    # a 128^3 block with the 15x15x41 PSF
    ],
)
def test_convolve_inplace_matches_oracle(cuda, shape, kshape):
    out, ref = conv_case(cuda, shape, kshape)
    assert rel_max(out, ref) < TOL, (rel_max(out, ref), rel_l2(out, ref))


def test_convolve_repeated_kernel_uses_cache_and_stays_exact(cuda):
    r = np.random.default_rng(7)
    k = S.gaussian_psf((1.5, 1.5, 4.0), (9, 9, 21), 30.0)
    for i in range(3):
        im = (r.random((30, 40, 50)) * 50).astype(np.float32)
        ref = O.conv_extended(im, k, O.MIRROR)
        out = im.copy()
        cuda.convolution3DfftCUDAInPlace(out, [30, 40, 50], k, list(k.shape), 0)
        assert rel_max(out, ref) < TOL


def test_errors_leave_image_unmodified(cuda):
    im = np.ones((8, 8, 8), dtype=np.float32)
    k = np.ones((4, 3, 3), dtype=np.float32)  # even size: rejected
    before = im.copy()
    cuda.convolution3DfftCUDAInPlace(im, [8, 8, 8], k, [4, 3, 3], 0)
    assert "odd" in cuda.last_error()
    np.testing.assert_array_equal(im, before)
    with pytest.raises(MvdError):
        cuda.convolve3d_inplace(im, [8, 8, 8], np.ones((3, 3, 3), np.float32), [3, 3, 3], 9999)
    np.testing.assert_array_equal(im, before)


def test_device_queries(cuda):
    n = cuda.getNumDevicesCUDA()
    assert n >= 1
    assert cuda.getCUDAcomputeCapabilityMajorVersion(0) >= 10
    assert cuda.getMemDeviceCUDA(0) > 0
    assert 0 < cuda.getFreeMemDeviceCUDA(0) <= cuda.getMemDeviceCUDA(0)
    assert len(cuda.getNameDeviceCUDA(0)) > 0
    assert cuda.lib.convolution3DfftCUDA(None, None, None, None, 0) is None or True
