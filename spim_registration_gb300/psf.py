"""Host-side mirror of ExtractPSF (spim/process/fusion/deconvolution/ExtractPSF.java) over the
library's PSF kernels: bead-neighbourhood extraction, normalisation and the transformation of
each view's PSF into the fused frame run on the GPU (mvd_extract_psf, mvd_transformed_psf_size,
mvd_transform_psf).  Volumes are numpy float32 arrays [z, y, x] (or CUDA tensors for the view);
bead locations are (x, y, z) in the view's pixel frame; models are row-packed 3x4 affines.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native


def _torch():
    import torch

    return torch


def extract_psf_local(img, locations_xyz, psf_size_xyz, normalize=False, device: int = 0) -> np.ndarray:
    """ExtractPSF.extractPSFLocal (:374-415), optionally followed by ExtractPSF.normalize (:298-316)."""
    torch = _torch()
    lib = native.load()
    t = img if getattr(img, "is_cuda", False) else torch.from_numpy(
        np.ascontiguousarray(img, dtype=np.float32)).to(f"cuda:{device}")
    loc = np.ascontiguousarray(np.asarray(locations_xyz, dtype=np.float64).reshape(-1, 3))
    px, py, pz = (int(s) for s in psf_size_xyz)
    out = torch.empty((pz, py, px), dtype=torch.float32, device=t.device)
    sz, sy, sx = t.shape
    st = torch.cuda.current_stream(t.device)
    native.check(lib.mvd_extract_psf(t.data_ptr(), native.iarr([sx, sy, sz]),
                                     loc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(loc),
                                     native.iarr([px, py, pz]), out.data_ptr(), int(bool(normalize)),
                                     t.device.index, ctypes.c_void_p(st.cuda_stream)))
    return out.cpu().numpy()


def transformed_psf_size(psf_size_xyz, model):
    """ExtractPSF.transformPSF (:325-372): (odd output size (x, y, z), offset)."""
    lib = native.load()
    dims = (ctypes.c_int * 3)()
    off = (ctypes.c_double * 3)()
    native.check(lib.mvd_transformed_psf_size(native.iarr(list(psf_size_xyz)),
                                              (ctypes.c_double * 12)(*np.asarray(model, dtype=np.float64).ravel()),
                                              dims, off))
    return tuple(dims), tuple(off)


def transform_psf(psf: np.ndarray, model, device: int = 0) -> np.ndarray:
    """ExtractPSF.transformPSF + transform (:325-372, :417-464): the PSF resampled by the view's
    model into an odd-sized box whose centre is the PSF's centre voxel."""
    torch = _torch()
    lib = native.load()
    psf = np.ascontiguousarray(psf, dtype=np.float32)
    pz, py, px = psf.shape
    (nx, ny, nz), off = transformed_psf_size((px, py, pz), model)
    t = torch.from_numpy(psf).to(f"cuda:{device}")
    out = torch.empty((nz, ny, nx), dtype=torch.float32, device=t.device)
    st = torch.cuda.current_stream(t.device)
    native.check(lib.mvd_transform_psf(t.data_ptr(), native.iarr([px, py, pz]),
                                       (ctypes.c_double * 12)(*np.asarray(model, dtype=np.float64).ravel()),
                                       native.iarr([nx, ny, nz]), (ctypes.c_double * 3)(*off), out.data_ptr(),
                                       device, ctypes.c_void_p(st.cuda_stream)))
    return out.cpu().numpy()


def make_same_size(img: np.ndarray, size_xyz) -> np.ndarray:
    """ExtractPSF.makeSameSize (:466-503): centred in a box of ``size_xyz``, the image's minimum
    outside it."""
    nx, ny, nz = size_xyz
    sz, sy, sx = img.shape
    out = np.full((nz, ny, nx), img.min(), dtype=img.dtype)
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    iz, iy, ix = z - nz // 2 + sz // 2, y - ny // 2 + sy // 2, x - nx // 2 + sx // 2
    ok = (iz >= 0) & (iy >= 0) & (ix >= 0) & (iz < sz) & (iy < sy) & (ix < sx)
    out[ok] = img[iz[ok], iy[ok], ix[ok]]
    return out


class ExtractPSF:
    """ExtractPSF: per view, the extracted PSF (normalised) and its transformed version."""

    def __init__(self, device: int = 0):
        self.device = device
        self.viewIds = []
        self.pointSpreadFunctions = {}
        self.originalPSFs = {}

    def extractNextImg(self, img, viewId, model, locations_xyz, psf_size_xyz):
        """ExtractPSF.extractNextImg (:277-296)."""
        original = extract_psf_local(img, locations_xyz, psf_size_xyz, normalize=True, device=self.device)
        self.viewIds.append(viewId)
        self.pointSpreadFunctions[viewId] = transform_psf(original, model, self.device)
        self.originalPSFs[viewId] = original

    def getPSFMap(self):
        return self.pointSpreadFunctions

    def getTransformedPSF(self, viewId):
        return self.pointSpreadFunctions[viewId]

    def getInputCalibrationPSFs(self):
        return self.originalPSFs

    def getViewIdsForPSFs(self):
        return self.viewIds

    def computeMaxDimTransformedPSF(self):
        """:523-539, (x, y, z)."""
        dims = np.array([p.shape[::-1] for p in self.pointSpreadFunctions.values()])
        return tuple(int(d) for d in dims.max(axis=0))

    def computeAverageTransformedPSF(self) -> np.ndarray:
        """:194-241: the transformed PSFs summed into a box of the largest size, each placed point-
        mirrored about the centres (loc -> psfCenter - loc + avgCenter, as the reference does)."""
        mx, my, mz = self.computeMaxDimTransformedPSF()
        avg = np.zeros((mz, my, mx), dtype=np.float32)
        ac = np.array([mz // 2, my // 2, mx // 2])
        for v in self.viewIds:
            p = self.pointSpreadFunctions[v]
            pc = np.array(p.shape) // 2
            z, y, x = np.meshgrid(*[np.arange(s) for s in p.shape], indexing="ij")
            tz, ty, tx = pc[0] - z + ac[0], pc[1] - y + ac[1], pc[2] - x + ac[2]
            ok = (tz >= 0) & (ty >= 0) & (tx >= 0) & (tz < mz) & (ty < my) & (tx < mx)
            np.add.at(avg, (tz[ok], ty[ok], tx[ok]), p[ok])
        return avg
