"""Host-side mirror of the reference's deconvolution classes over the sm_103a library.

The names, argument meanings and call order follow the Java classes they stand in for:

* ``CUDAFourierConvolution``  -- the JNA interface (spim/process/cuda/CUDAFourierConvolution.java:25-32,
  CUDAStandardFunctions.java:26-45): ``convolution3DfftCUDAInPlace(im, imDim, kernel, kernelDim, devCUDA)``
  with ``imDim``/``kernelDim`` reversed ({z, y, x}) as MVDeconFFTThreads.getCUDACoordinates does.
* ``PSFTYPE``, ``MVDeconFFT``, ``MVDeconInput``, ``MVDeconvolution`` -- the iteration engine
  (spim/process/fusion/deconvolution/MVDeconFFT.java:47-172, MVDeconInput.java:31-80,
  MVDeconvolution.java:94-211, 349-465).  ``MVDeconvolution(views, iterationType, numIterations,
  lambda, osemspeedup, osemspeedupindex, name)`` runs the whole deconvolution in its constructor,
  like the Java one; ``getPsi()`` returns the masked result.

Images are numpy float32 arrays in [z, y, x] order (x fastest: the ArrayImg layout).
"""
from __future__ import annotations

import ctypes
import enum

import numpy as np

from . import native


class PSFTYPE(enum.IntEnum):
    """MVDeconFFT.PSFTYPE (MVDeconFFT.java:49)."""

    OPTIMIZATION_II = 0
    OPTIMIZATION_I = 1
    EFFICIENT_BAYESIAN = 2
    INDEPENDENT = 3


FLAG_PLAIN = 1
FLAG_NO_GRAPH = 2
FLAG_AUTOTUNE = 4
FLAG_TENSOR_DFT = 8  # middle 16-point DFTs of the 320 / 288 z passes on the tensor cores


def FLAG_REF_SUM_THREADS(threads: int) -> int:
    """MVD_FLAG_REF_SUM_THREADS(t): normalise the kernels as AdjustInput.sumImg does with t
    threads (portion 0 of divideIntoPortions(n, 2 t) counted twice, AdjustInput.java:114-118)."""
    if not 1 <= int(threads) <= 32767:
        raise ValueError("threads must be in [1, 32767]")
    return int(threads) << 16


class CUDAFourierConvolution:
    """The JNA interface bound to libFourierConvolutionCUDA (CUDAFourierConvolution.java:25-32)."""

    def __init__(self, path: str | None = None):
        self.lib = native.load(path)

    # CUDAStandardFunctions
    def getNumDevicesCUDA(self) -> int:
        return self.lib.getNumDevicesCUDA()

    def getNameDeviceCUDA(self, devCUDA: int) -> str:
        buf = ctypes.create_string_buffer(256)
        self.lib.getNameDeviceCUDA(devCUDA, buf)
        return buf.value.decode(errors="replace")

    def getMemDeviceCUDA(self, devCUDA: int) -> int:
        return self.lib.getMemDeviceCUDA(devCUDA)

    def getFreeMemDeviceCUDA(self, devCUDA: int) -> int:
        return self.lib.getFreeMemDeviceCUDA(devCUDA)

    def getCUDAcomputeCapabilityMajorVersion(self, devCUDA: int) -> int:
        return self.lib.getCUDAcomputeCapabilityMajorVersion(devCUDA)

    def getCUDAcomputeCapabilityMinorVersion(self, devCUDA: int) -> int:
        return self.lib.getCUDAcomputeCapabilityMinorVersion(devCUDA)

    # CUDAFourierConvolution
    def convolution3DfftCUDAInPlace(self, im: np.ndarray, imDim, kernel: np.ndarray, kernelDim, devCUDA: int):
        """In-place convolution; `im` is modified.  Errors are reported like the Java side sees
        them (void return): the image is left unmodified and the message is kept."""
        self.lib.convolution3DfftCUDAInPlace(native.fptr(im), native.iarr(imDim), native.fptr(kernel),
                                             native.iarr(kernelDim), devCUDA)

    def convolve3d_inplace(self, im: np.ndarray, imDim, kernel: np.ndarray, kernelDim, devCUDA: int = 0):
        """Status-checked variant (raises MvdError)."""
        native.check(self.lib.mvd_convolve3d_inplace(native.fptr(im), native.iarr(imDim), native.fptr(kernel),
                                                     native.iarr(kernelDim), devCUDA))

    def last_error(self) -> str:
        return self.lib.mvd_last_error().decode(errors="replace")


class MVDeconFFT:
    """One view: observed image, weight and PSF (kernel1), as MVDeconFFT (MVDeconFFT.java:79-172)."""

    def __init__(self, image: np.ndarray, weight: np.ndarray, kernel: np.ndarray, deviceList=(0,),
                 useBlocks: bool = False, blockSize=None, saveMemory: bool = False):
        self.image = np.ascontiguousarray(image, dtype=np.float32)
        self.weight = np.ascontiguousarray(weight, dtype=np.float32)
        self.kernel1 = np.ascontiguousarray(kernel, dtype=np.float32)
        if any(s % 2 == 0 for s in self.kernel1.shape):
            raise ValueError("kernel sizes must be odd")
        if self.image.shape != self.weight.shape:
            raise ValueError("image and weight differ in size")
        self.deviceList = list(deviceList)
        self.useBlocks = useBlocks
        self.blockSize = tuple(blockSize) if blockSize is not None else None
        self.numViews = 0

    def getImage(self):
        return self.image

    def getWeight(self):
        return self.weight

    def getKernel1(self):
        return self.kernel1


class MVDeconInput:
    """The list of views (MVDeconInput.java:31-80)."""

    def __init__(self):
        self.views: list[MVDeconFFT] = []

    def add(self, view: MVDeconFFT):
        self.views.append(view)
        for v in self.views:
            v.numViews = len(self.views)

    def getViews(self):
        return self.views

    def getNumViews(self):
        return len(self.views)


def _input_array(a):
    """A view or weight volume: a numpy array (host) or a contiguous float32 CUDA tensor (device,
    e.g. from ``inputs.transform_input``), which mvd_create copies without a host round trip."""
    if getattr(a, "is_cuda", False):
        if str(a.dtype) != "torch.float32" or not a.is_contiguous():
            raise ValueError("device volumes must be contiguous float32 tensors")
        return a
    return np.ascontiguousarray(a, dtype=np.float32)


def _input_ptr(a):
    if isinstance(a, np.ndarray):
        return native.fptr(a)
    return ctypes.cast(ctypes.c_void_p(a.data_ptr()), native._F)


class Deconvolution:
    """Handle over the library's whole-deconvolution API (mvd_create / mvd_run_* / mvd_get_psi).

    views and weights are numpy arrays or float32 CUDA tensors on ``device`` ([z, y, x])."""

    def __init__(self, views, weights, psfs, psftype: int, lam: float, device: int = 0, flags: int = 0,
                 block=None):
        self.lib = native.load()
        views = [_input_array(v) for v in views]
        weights = [_input_array(w) for w in weights]
        psfs = [np.ascontiguousarray(p, dtype=np.float32) for p in psfs]
        if not views:
            raise ValueError("no views")
        shape = tuple(views[0].shape)
        for a in views + weights:
            if tuple(a.shape) != shape:
                raise ValueError("all views and weights must share one shape")
        self.shape = shape
        self.n_views = len(views)
        self._keep = (views, weights, psfs)
        if any(not isinstance(a, np.ndarray) for a in views + weights):
            import torch  # device inputs: the work that wrote them must be complete

            torch.cuda.synchronize(device)
        nz, ny, nx = shape
        vp = (native._F * self.n_views)(*[_input_ptr(v) for v in views])
        wp = (native._F * self.n_views)(*[_input_ptr(w) for w in weights])
        pp = (native._F * self.n_views)(*[native.fptr(p) for p in psfs])
        pd = []
        for p in psfs:
            kz, ky, kx = p.shape
            pd += [kx, ky, kz]
        h = native._H()
        blk = native.iarr(block) if block is not None else None
        native.check(self.lib.mvd_create(ctypes.byref(h), device, native.iarr([nx, ny, nz]), self.n_views, vp, wp, pp,
                                         native.iarr(pd), int(psftype), float(lam), int(flags), blk))
        self.h = h
        self.psf_shapes = [p.shape for p in psfs]

    def close(self):
        if getattr(self, "h", None):
            self.lib.mvd_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run_view(self, v: int):
        native.check(self.lib.mvd_run_view(self.h, v))

    def run_iteration(self):
        native.check(self.lib.mvd_run_iteration(self.h))

    def run(self, iterations: int):
        native.check(self.lib.mvd_run(self.h, iterations))

    def synchronize(self):
        native.check(self.lib.mvd_synchronize(self.h))

    def get_psi(self, masked: bool = False, out: np.ndarray | None = None) -> np.ndarray:
        """psi as float32 [z, y, x]; ``out`` may be a caller-owned (e.g. pinned) array to fill."""
        if out is None:
            out = np.empty(self.shape, dtype=np.float32)
        elif out.shape != tuple(self.shape) or out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous float32 array of psi's shape")
        native.check(self.lib.mvd_get_psi(self.h, native.fptr(out), 1 if masked else 0))
        return out

    def set_psi(self, psi: np.ndarray):
        psi = np.ascontiguousarray(psi, dtype=np.float32)
        if psi.shape != self.shape:
            raise ValueError("psi has the wrong shape")
        native.check(self.lib.mvd_set_psi(self.h, native.fptr(psi)))

    def initial_average(self) -> float:
        d = ctypes.c_double()
        native.check(self.lib.mvd_get_initial_average(self.h, ctypes.byref(d)))
        return d.value

    def kernel(self, view: int, which: int) -> np.ndarray:
        out = np.empty(self.psf_shapes[view], dtype=np.float32)
        native.check(self.lib.mvd_get_kernel(self.h, view, which, native.fptr(out)))
        return out

    def stats(self, iteration: int, view: int):
        s, m = ctypes.c_double(), ctypes.c_double()
        native.check(self.lib.mvd_get_stats(self.h, iteration, view, ctypes.byref(s), ctypes.byref(m)))
        return s.value, m.value

    def iteration(self) -> int:
        i = ctypes.c_int()
        native.check(self.lib.mvd_get_iteration(self.h, ctypes.byref(i)))
        return i.value

    def stream(self) -> int:
        """cudaStream_t (as an integer) the handle enqueues on."""
        v = ctypes.c_void_p()
        native.check(self.lib.mvd_get_stream(self.h, ctypes.byref(v)))
        return int(v.value or 0)

    def launch_count(self) -> int:
        n = ctypes.c_longlong()
        native.check(self.lib.mvd_get_launch_count(self.h, ctypes.byref(n)))
        return n.value

    def profile_iteration(self):
        """One eager iteration with per-pass CUDA events: {kind: (ms, launches)}."""
        ms = (ctypes.c_double * 5)()
        ln = (ctypes.c_int * 5)()
        native.check(self.lib.mvd_profile_iteration(self.h, ms, ln))
        names = ["plane_fwd", "zpass", "plane_inv_quotient", "plane_inv_update", "other"]
        return {n: (ms[i], ln[i]) for i, n in enumerate(names)}

    def forward(self) -> float:
        """Poisson NLL of the image-formation model at the current psi and kernel1 (FP64)."""
        d = ctypes.c_double()
        native.check(self.lib.mvd_forward(self.h, ctypes.byref(d)))
        return d.value

    def backward(self):
        """(dNLL/dpsi, [dNLL/dkernel1_v]) at the current psi and kernel1."""
        g = np.empty(self.shape, dtype=np.float32)
        gk = [np.empty(s, dtype=np.float32) for s in self.psf_shapes]
        ptrs = (native._F * self.n_views)(*[native.fptr(a) for a in gk])
        native.check(self.lib.mvd_backward(self.h, native.fptr(g), ptrs))
        return g, gk

    def set_kernel(self, view: int, which: int, data: np.ndarray):
        data = np.ascontiguousarray(data, dtype=np.float32)
        if data.shape != self.psf_shapes[view]:
            raise ValueError("kernel has the wrong shape")
        native.check(self.lib.mvd_set_kernel(self.h, view, which, native.fptr(data)))

    def plan(self, view: int):
        t, s, e = (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
        pv = ctypes.c_longlong()
        native.check(self.lib.mvd_get_plan(self.h, view, t, s, e, ctypes.byref(pv)))
        th, var = ctypes.c_int(), ctypes.c_int()
        native.check(self.lib.mvd_get_plan_variant(self.h, view, ctypes.byref(th), ctypes.byref(var)))
        return dict(tiles=tuple(t), tile=tuple(s), effective=tuple(e), padded_voxels=pv.value,
                    threads=th.value, kernels="compiled" if var.value & 1 else "generic",
                    radix_order="ascending" if var.value & 2 else "descending",
                    tensor_dft=bool(var.value & 4), staged=bool(var.value & 8))


class MVDeconvolution:
    """MVDeconvolution (MVDeconvolution.java:94-211): runs all iterations in the constructor.

    ``osemspeedup``/``osemspeedupindex`` are accepted for signature compatibility; as in the
    reference they only matter for the weight preparation, which happens before this class.
    """

    minValue = np.float32(1e-4)

    def __init__(self, views: MVDeconInput, iterationType: PSFTYPE, numIterations: int, lam: float,
                 osemspeedup: float = 1.0, osemspeedupindex: int = 0, name: str = "", device: int | None = None,
                 flags: int = 0, initialImage: np.ndarray | None = None):
        data = views.getViews()
        self.name = name
        self.views = views
        self.numIterations = numIterations
        dev = device if device is not None else data[0].deviceList[0]
        blk = data[0].blockSize if data[0].useBlocks else None
        self.handle = Deconvolution([d.image for d in data], [d.weight for d in data], [d.kernel1 for d in data],
                                    int(iterationType), lam, dev, flags, blk)
        if initialImage is not None:
            # MVDeconvolution.loadInitialImage (:258-341): values <= 0 become minValue
            init = np.asarray(initialImage, dtype=np.float32)
            self.handle.set_psi(np.where(init <= 0, self.minValue, init).astype(np.float32))
        self.i = 0
        while self.i < numIterations:
            self.runIteration()
        self.psi = self.handle.get_psi(masked=True)

    def runIteration(self):
        self.handle.run_iteration()
        self.i += 1

    def getPsi(self):
        return self.psi

    def getCurrentIteration(self):
        return self.i
