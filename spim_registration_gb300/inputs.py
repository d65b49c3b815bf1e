"""Input preparation of the deconvolution on the GPU: the host-side mirror of the reference's
TransformInput / TransformInputAndWeights / TransformWeights (spim/process/fusion/deconvolution/,
TransformInput.java:90-116, BlendingRealRandomAccess.java:91-121), WeightNormalizer
(WeightNormalizer.java:73-253) and ProcessForDeconvolution.adjustForOSEM (:372-405).

Volumes are float32 CUDA tensors in [z, y, x] order on one device; every call enqueues on the
torch current stream of that device, so the prepared views and weights can go straight into
``Deconvolution`` without a host round trip.  Affine transforms are the view registrations
(view -> world) as a 3x4 row-major matrix, the imglib2 AffineTransform3D layout.
"""
from __future__ import annotations

import ctypes
import enum
import os

import numpy as np

from . import native


class WeightType(enum.IntEnum):
    """The two normalisations of ProcessForDeconvolution.WeightType that rescale weights."""

    VIRTUAL_WEIGHTS = 0
    PRECOMPUTED_WEIGHTS = 1


def _torch():
    import torch

    return torch


def _stream(t):
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _device_volume(a, device):
    torch = _torch()
    if isinstance(a, np.ndarray):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(f"cuda:{device}")
    if a.dtype != torch.float32 or not a.is_cuda:
        raise ValueError("volumes must be float32 (numpy or CUDA tensors)")
    return a.contiguous()


def transform_input(view, affine, offset_xyz, box_shape_zyx, border_xyz=None, blending_xyz=None, device: int = 0,
                    image: bool = True):
    """One view resampled into the fused box (TransformInput) and, when ``border_xyz`` and
    ``blending_xyz`` are given, its cosine blending weight (TransformWeights); both at once is
    TransformInputAndWeights.  Box voxel (x, y, z) sits at world position (x, y, z) +
    ``offset_xyz``.  Returns ``(image, weight)`` CUDA tensors (``None`` for the one not asked)."""
    torch = _torch()
    lib = native.load()
    v = _device_volume(view, device)
    a = np.asarray(affine, dtype=np.float64).reshape(-1)
    if a.size != 12:
        raise ValueError("affine must be 3x4")
    want_w = border_xyz is not None and blending_xyz is not None
    out_i = torch.empty(tuple(box_shape_zyx), dtype=torch.float32, device=v.device) if image else None
    out_w = torch.empty(tuple(box_shape_zyx), dtype=torch.float32, device=v.device) if want_w else None
    nz, ny, nx = box_shape_zyx
    sz, sy, sx = v.shape
    st = lib.mvd_transform_view(v.data_ptr(), native.iarr([sx, sy, sz]), (ctypes.c_double * 12)(*a),
                                native.iarr([int(o) for o in offset_xyz]), native.iarr([nx, ny, nz]),
                                out_i.data_ptr() if out_i is not None else None,
                                out_w.data_ptr() if out_w is not None else None,
                                (ctypes.c_float * 3)(*border_xyz) if want_w else None,
                                (ctypes.c_float * 3)(*blending_xyz) if want_w else None, v.device.index, _stream(v))
    native.check(st)
    return out_i, out_w


class WeightNormalizer:
    """WeightNormalizer (WeightNormalizer.java:50-130) over device weight volumes: ``process()``
    computes the overlap statistics; ``apply(osem)`` normalises in place (VIRTUAL or PRECOMPUTED)
    with the OSEM factor of ProcessForDeconvolution.adjustForOSEM folded in."""

    def __init__(self, weights, weight_type: WeightType = WeightType.VIRTUAL_WEIGHTS, num_portions: int | None = None):
        if not weights:
            raise ValueError("no weights")
        self.weights = list(weights)
        self.weight_type = WeightType(weight_type)
        shape = tuple(self.weights[0].shape)
        if any(tuple(w.shape) != shape for w in self.weights):
            raise ValueError("weights must share one shape")
        self.n = int(np.prod(shape))
        # the reference splits the volume into 2 x its thread count portions
        self.num_portions = int(num_portions or 2 * (os.cpu_count() or 1))
        self.minOverlappingViews = len(self.weights)
        self.avgOverlappingViews = 0.0

    def _ptrs(self):
        return (ctypes.c_void_p * len(self.weights))(*[w.data_ptr() for w in self.weights])

    def process(self) -> bool:
        lib = native.load()
        mn = ctypes.c_int()
        avg = ctypes.c_double()
        w0 = self.weights[0]
        native.check(lib.mvd_weight_overlap(self._ptrs(), len(self.weights), self.n, min(self.num_portions, self.n),
                                            ctypes.byref(mn), ctypes.byref(avg), w0.device.index, _stream(w0)))
        self.minOverlappingViews, self.avgOverlappingViews = mn.value, avg.value
        return True

    def getMinOverlappingViews(self) -> int:
        return self.minOverlappingViews

    def getAvgOverlappingViews(self) -> float:
        return self.avgOverlappingViews

    def osem_speedup(self, osem_index: int, manual: float = 1.0) -> float:
        """ProcessForDeconvolution (:349-356): 0 -> 1, 1 -> min overlap, 2 -> average overlap,
        3 -> the manual value; overlaps below 1 are raised to 1."""
        if osem_index == 1:
            return float(max(1, self.minOverlappingViews))
        if osem_index == 2:
            return max(1.0, self.avgOverlappingViews)
        if osem_index == 3:
            return float(manual)
        return 1.0

    def apply(self, osem: float = 1.0):
        lib = native.load()
        w0 = self.weights[0]
        native.check(lib.mvd_normalize_weights(self._ptrs(), len(self.weights), self.n, float(osem),
                                               int(self.weight_type), w0.device.index, _stream(w0)))
        return self.weights
