"""Host-side mirror of the difference-of-Gaussian detector's separable-convolution interface.

* ``CUDASeparableConvolution`` -- the JNA interface (spim/process/cuda/CUDASeparableConvolution.java:34-46):
  ``convolve_K(image, kernelX, kernelY, kernelZ, w, h, d, convolveX, convolveY, convolveZ,
  outofbounds, outofboundsvalue, devCUDA)`` for K in {7, 15, 31, 63, 127}, in place on a float32
  array, and ``convolutionCPU`` (computed on GPU 0: the library has no CPU path).
* ``CUDASeparableConvolutionFunctions`` -- the Java helper (CUDASeparableConvolutionFunctions.java:32-266):
  ``gauss(img, dim, sigma, oobs, oobsValue)`` builds the Gaussian kernels, centres them in the
  smallest supported size and calls ``convolve_K``.

Gaussian kernels follow mpicbg's ``Util.createGaussianKernel1DDouble`` (the mpicbg library, a
dependency the reference does not vendor), restated from its published behaviour: for sigma <= 0
the 3-tap identity, else 2 * (int)(3 sigma + 0.5) + 1 taps (at least 3) of exp(-x^2 / (2 sigma^2))
centred at size / 2, optionally normalised to unit sum.
"""
from __future__ import annotations

import ctypes
import enum

import numpy as np

from . import native

SUPPORTED_KERNEL_SIZES = (7, 15, 31, 63, 127)


class OutOfBounds(enum.IntEnum):
    """CUDASeparableConvolutionFunctions.OutOfBounds (:34); the ordinal goes to the library."""

    ZERO = 0
    VALUE = 1
    EXTEND_BORDER_PIXELS = 2


def create_gaussian_kernel_1d_double(sigma: float, normalize: bool) -> np.ndarray:
    if sigma <= 0:
        k = np.zeros(3)
        k[1] = 1.0
    else:
        size = max(3, 2 * int(3 * sigma + 0.5) + 1)
        two_sq_sigma = 2 * sigma * sigma
        x = np.arange(size) - size // 2
        k = np.exp(-(x * x) / two_sq_sigma)
    if normalize:
        k = k / k.sum()
    return k


def get_float_kernel_padded(kernel: np.ndarray, size: int) -> np.ndarray | None:
    """CUDASeparableConvolutionFunctions.getFloatKernelPadded (:253-265)."""
    if len(kernel) > size:
        return None
    k = np.zeros(size, dtype=np.float32)
    s = (size - len(kernel)) // 2
    k[s:s + len(kernel)] = np.asarray(kernel, dtype=np.float64).astype(np.float32)
    return k


def get_cuda_kernels(sigma, supported=SUPPORTED_KERNEL_SIZES):
    """CUDASeparableConvolutionFunctions.getCUDAKernels (:225-251): normalised Gaussians centred in
    the smallest supported size that holds the longest of them; None when none does."""
    kernels = [create_gaussian_kernel_1d_double(s, True) for s in sigma]
    longest = max(len(k) for k in kernels)
    fits = [s for s in supported if longest <= s]
    if not fits:
        return None
    size = min(fits)
    return [get_float_kernel_padded(k, size) for k in kernels]


def _fp(a):
    return None if a is None else native.fptr(a)


class CUDASeparableConvolution:
    """The JNA interface over the library (the same .so as the deconvolution)."""

    def __init__(self):
        self.lib = native.load()

    def _convolve(self, K, image, kx, ky, kz, w, h, d, cx, cy, cz, oob, value, dev) -> bool:
        if image.dtype != np.float32 or not image.flags.c_contiguous or image.size != w * h * d:
            raise ValueError("image must be a contiguous float32 array of w * h * d values")
        ks = [None if k is None else np.ascontiguousarray(k, dtype=np.float32) for k in (kx, ky, kz)]
        for k in ks:
            if k is not None and k.size != K:
                raise ValueError(f"kernels of convolve_{K} have {K} taps")
        fn = getattr(self.lib, f"convolve_{K}")
        return bool(fn(native.fptr(image), _fp(ks[0]), _fp(ks[1]), _fp(ks[2]), w, h, d, int(cx), int(cy), int(cz),
                       int(oob), float(value), int(dev)))

    def convolve_127(self, *a) -> bool:
        return self._convolve(127, *a)

    def convolve_63(self, *a) -> bool:
        return self._convolve(63, *a)

    def convolve_31(self, *a) -> bool:
        return self._convolve(31, *a)

    def convolve_15(self, *a) -> bool:
        return self._convolve(15, *a)

    def convolve_7(self, *a) -> bool:
        return self._convolve(7, *a)

    def convolutionCPU(self, image, kx, ky, kz, rx, ry, rz, w, h, d, oob, value):
        ks = [np.ascontiguousarray(k, dtype=np.float32) for k in (kx, ky, kz)]
        self.lib.convolutionCPU(native.fptr(image), *[native.fptr(k) for k in ks], rx, ry, rz, w, h, d, int(oob),
                                float(value))


class CUDASeparableConvolutionFunctions:
    """CUDASeparableConvolutionFunctions: Gaussian smoothing through the library."""

    def __init__(self, cuda: CUDASeparableConvolution | None = None, cudaDeviceId: int = 0):
        self.cuda = cuda or CUDASeparableConvolution()
        self.cudaDeviceId = cudaDeviceId

    def gauss(self, img: np.ndarray, dim, sigma, oobs=OutOfBounds.EXTEND_BORDER_PIXELS, oobsValue: float = 0.0) -> bool:
        """In place on ``img`` (flat or shaped float32, x fastest); ``dim`` = [w] / [w, h] / [w, h, d];
        ``sigma`` a number or one per dimension (:123-210)."""
        if img is None or dim is None or sigma is None:
            return False
        n = len(dim)
        if n == 0 or n > 3:
            return False
        if np.isscalar(sigma):
            sigma = [float(sigma)] * n
        if len(sigma) != n:
            return False
        kernels = get_cuda_kernels(sigma)
        if kernels is None:
            return False
        size = len(kernels[0])
        w = dim[0]
        h = dim[1] if n > 1 else 1
        d = dim[2] if n > 2 else 1
        ks = kernels + [None] * (3 - n)
        flat = img.reshape(-1)
        if not np.shares_memory(flat, img):
            raise ValueError("img must be contiguous")
        return getattr(self.cuda, f"convolve_{size}")(flat, ks[0], ks[1], ks[2], w, h, d, ks[0] is not None,
                                                     ks[1] is not None, ks[2] is not None, int(oobs), oobsValue,
                                                     self.cudaDeviceId)
