"""Separable convolution library (convolve_K / convolutionCPU / the device entry point) against
the oracle on the GPU.  FP32 accumulation of up to 127 taps per pass: max abs error <= 2e-6 of
the output's max abs value."""
import numpy as np
import pytest

from oracle import mvdecon_oracle as O
from spim_registration_gb300 import native
from spim_registration_gb300.separable import (CUDASeparableConvolution, CUDASeparableConvolutionFunctions,
                                               OutOfBounds, get_cuda_kernels)

pytestmark = pytest.mark.gpu
TOL = 2e-6


def _close(got, want):
    scale = max(float(np.abs(want).max()), 1e-30)
    err = float(np.abs(got.astype(np.float64) - want).max()) / scale
    assert err <= TOL, err


@pytest.mark.parametrize("K", [7, 15, 31, 63, 127])
@pytest.mark.parametrize("oob", [0, 1, 2])
def test_convolve_k_matches_oracle(K, oob):
    rng = np.random.default_rng(K * 10 + oob)
    img = (rng.random((23, 29, 37)) * 10).astype(np.float32)  # d, h, w
    ks = [rng.standard_normal(K).astype(np.float32) for _ in range(3)]  # asymmetric taps
    want = O.separable_convolve(img, ks, oob, 1.5)
    cuda = CUDASeparableConvolution()
    got = img.copy()
    assert getattr(cuda, f"convolve_{K}")(got.reshape(-1), *ks, 37, 29, 23, True, True, True, oob, 1.5, 0)
    _close(got, want)


@pytest.mark.parametrize("flags", [(1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (0, 1, 1)])
def test_axis_flags(flags):
    rng = np.random.default_rng(sum(f << i for i, f in enumerate(flags)))
    img = rng.random((70, 66, 515)).astype(np.float32)  # two x segments, two axis chunks
    ks = [rng.standard_normal(15).astype(np.float32) for _ in range(3)]
    want = O.separable_convolve(img, [k if f else None for k, f in zip(ks, flags)], 2)
    got = img.copy()
    assert CUDASeparableConvolution().convolve_15(got.reshape(-1), ks[0] if flags[0] else None,
                                                  ks[1] if flags[1] else None, ks[2] if flags[2] else None,
                                                  515, 66, 70, *flags, 2, 0.0, 0)
    _close(got, want)


@pytest.mark.parametrize("shape", [(1, 1, 301), (1, 40, 33), (5, 3, 2), (130, 1, 1)])
def test_one_two_three_dimensional_and_tiny_images(shape):
    rng = np.random.default_rng(sum(shape))
    img = rng.random(shape).astype(np.float32)
    ks = [rng.standard_normal(63).astype(np.float32) for _ in range(3)]  # halo wider than the image
    d, h, w = shape
    flags = (True, h > 1, d > 1)
    for oob in (0, 1, 2):
        want = O.separable_convolve(img, [k if f else None for k, f in zip(ks, flags)], oob, -0.5)
        got = img.copy()
        assert CUDASeparableConvolution().convolve_63(got.reshape(-1), ks[0], ks[1] if flags[1] else None,
                                                      ks[2] if flags[2] else None, w, h, d, *flags, oob, -0.5, 0)
        _close(got, want)


def test_gauss_of_the_java_helper():
    rng = np.random.default_rng(5)
    img = (rng.random((48, 64, 80)) * 100).astype(np.float32)
    sigma = [1.8, 1.8, 3.2]
    ks = get_cuda_kernels(sigma)
    want = O.separable_convolve(img, ks, O.SEP_EXTEND)
    got = img.copy()
    assert CUDASeparableConvolutionFunctions(cudaDeviceId=0).gauss(got, [80, 64, 48], sigma)
    _close(got, want)
    # 2D and 1D forms of gauss (dim of length 2 / 1)
    plane = img[0].copy()
    want2 = O.separable_convolve(plane, get_cuda_kernels([2.0, 2.0]), O.SEP_EXTEND)
    assert CUDASeparableConvolutionFunctions().gauss(plane, [80, 64], 2.0)
    _close(plane, want2)


def test_convolution_cpu_entry_runs_the_same_passes():
    rng = np.random.default_rng(6)
    img = rng.random((20, 30, 40)).astype(np.float32)
    ks = [rng.standard_normal(2 * r + 1).astype(np.float32) for r in (2, 5, 0)]
    want = O.separable_convolve(img, ks, 1, 0.25)
    got = img.copy()
    CUDASeparableConvolution().convolutionCPU(got.reshape(-1), *ks, 2, 5, 0, 40, 30, 20, 1, 0.25)
    _close(got, want)


def test_device_entry_point_and_result_buffer():
    torch = pytest.importorskip("torch")
    lib = native.load()
    rng = np.random.default_rng(7)
    img = rng.random((33, 41, 57)).astype(np.float32)
    ks = [rng.standard_normal(n).astype(np.float32) for n in (9, 31, 5)]
    for use in [(1, 1, 1), (1, 1, 0)]:
        a = torch.from_numpy(img.copy()).cuda()
        b = torch.empty_like(a)
        kp = (native._F * 3)(*[native.fptr(k) if u else None for k, u in zip(ks, use)])
        res = native.ctypes.c_void_p()
        native.check(lib.mvd_separable_convolve_device(a.data_ptr(), b.data_ptr(), kp, native.iarr([9, 31, 5]),
                                                       native.iarr([57, 41, 33]), 2, 0.0, 0, None,
                                                       native.ctypes.byref(res)))
        torch.cuda.synchronize()
        out = (a if res.value == a.data_ptr() else b).cpu().numpy()
        assert res.value == (b.data_ptr() if sum(use) % 2 else a.data_ptr())
        _close(out, O.separable_convolve(img, [k if u else None for k, u in zip(ks, use)], 2))


def test_invalid_arguments_leave_the_image_unchanged():
    img = np.ones((4, 4, 4), dtype=np.float32)
    k = np.ones(7, dtype=np.float32)
    cuda = CUDASeparableConvolution()
    assert not cuda.convolve_7(img.reshape(-1), k, k, k, 4, 4, 4, True, True, True, 3, 0.0, 0)  # unknown oob
    assert not cuda.convolve_7(img.reshape(-1), k, k, k, 4, 4, 4, True, True, True, 2, 0.0, 99)  # no such device
    assert not cuda.lib.convolve_7(native.fptr(img.reshape(-1)), None, native.fptr(k), native.fptr(k), 4, 4, 4, 1, 1,
                                   1, 2, 0.0, 0)  # x requested without its kernel
    np.testing.assert_array_equal(img, 1.0)
    assert OutOfBounds.EXTEND_BORDER_PIXELS == 2
