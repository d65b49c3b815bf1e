"""FP64 restatement of the oracle's deconvolution in torch, for full-size checks.  TEST
INFRASTRUCTURE ONLY: used by ``tests/`` and by the accuracy check of ``bench.py`` (outside
its timed region), never by the library.

``mvdecon_oracle.Deconvolution(..., arith="f64")`` is the reference loop restated in numpy.  At
the benchmark's sizes (4 views of 512x512x256 with 31x31x61 PSFs) ten iterations of it take
many minutes on the host, so this module runs the same arithmetic in float64 with torch on
whatever device its tensors live on (a GPU for the full-size tests, the CPU for the pinning
test ``tests/test_oracle.py::test_fp64_torch_restatement_matches_the_numpy_oracle``).  The
kernels (``MVDeconFFT.init``) are PSF-sized and come from the numpy oracle itself.

Each convolution is the linear convolution of the extended image with the centred kernel,
cropped to the image (MVDeconFFT.java:384-560, MVDeconFFTThreads.java:39-70): the extended
image (``n + k - 1`` per axis) is zero-padded to a fast FFT length L >= n + k - 1, multiplied
by the kernel's spectrum at L and inverted; positions [k - 1, k - 1 + n) see no wrap-around.
This is ``mvdecon_oracle.conv_extended`` with a smaller (still exact) padding.
"""
from __future__ import annotations

import numpy as np
import torch

from oracle import mvdecon_oracle as O


def _fast_len(n: int) -> int:
    """Smallest 2,3,5,7-smooth length >= n."""
    m = max(1, n)
    while True:
        k = m
        for f in (2, 3, 5, 7):
            while k % f == 0:
                k //= f
        if k == 1:
            return m
        m += 1


def _mirror_index(n: int, lo: int, hi: int, device) -> torch.Tensor:
    idx = np.arange(-lo, n + hi)
    return torch.as_tensor(O.mirror_single_index(idx, n), device=device, dtype=torch.long)


def extend(img: torch.Tensor, lo, hi, mode: int, value: float = 0.0) -> torch.Tensor:
    """Views.extendMirrorSingle / Views.extendValue over [-lo, n + hi) per axis (z, y, x)."""
    if mode == O.MIRROR:
        out = img
        for d in range(3):
            out = torch.index_select(out, d, _mirror_index(img.shape[d], lo[d], hi[d], img.device))
        return out
    pad = (lo[2], hi[2], lo[1], hi[1], lo[0], hi[0])
    return torch.nn.functional.pad(img, pad, mode="constant", value=float(value))


class Convolver:
    """Convolutions of n-sized volumes with one kernel (kernel spectrum kept)."""

    def __init__(self, shape_zyx, kernel: np.ndarray, device):
        self.k = tuple(kernel.shape)
        self.n = tuple(shape_zyx)
        self.h = [s // 2 for s in self.k]
        self.hi = [s - 1 - s // 2 for s in self.k]
        self.L = [_fast_len(self.n[d] + self.k[d] - 1) for d in range(3)]
        kt = torch.as_tensor(np.asarray(kernel, dtype=np.float64), device=device)
        self.K = torch.fft.rfftn(kt, s=self.L)

    def __call__(self, img: torch.Tensor, mode: int, value: float = 0.0) -> torch.Tensor:
        ext = extend(img, self.hi, self.h, mode, value)
        full = torch.fft.irfftn(torch.fft.rfftn(ext, s=self.L) * self.K, s=self.L)
        k, n = self.k, self.n
        return full[k[0] - 1:k[0] - 1 + n[0], k[1] - 1:k[1] - 1 + n[1], k[2] - 1:k[2] - 1 + n[2]].contiguous()


def first_iteration_average(views) -> float:
    """FirstIteration.call (FirstIteration.java:84-154) in float64: the mean over voxels with a
    positive view value of the per-voxel mean of the positive values (0.5 if there are none)."""
    s = torch.zeros_like(views[0])
    c = torch.zeros_like(views[0])
    for v in views:
        pos = v > 0
        s += torch.where(pos, v, torch.zeros_like(v))
        c += pos.to(v.dtype)
    has = c > 0
    count = int(has.sum().item())
    if count == 0:
        return 0.5
    avg = float((s[has] / c[has]).sum().item()) / count
    return 0.5 if avg != avg else avg


class Deconvolution:
    """``mvdecon_oracle.Deconvolution`` in float64 (one whole-image block), on ``device``."""

    def __init__(self, views, weights, psfs, psftype, lam, device="cuda", quirk_threads=None):
        self.device = torch.device(device)
        dd = dict(device=self.device, dtype=torch.float64)
        self.views = [torch.as_tensor(np.asarray(v, dtype=np.float32)).to(**dd) for v in views]
        self.weights = [torch.as_tensor(np.asarray(w, dtype=np.float32)).to(**dd) for w in weights]
        self.lam = float(lam)
        k1, k2 = O.prepare_kernels(psfs, psftype, quirk_threads, "f64")
        shape = tuple(self.views[0].shape)
        self.c1 = [Convolver(shape, k, self.device) for k in k1]
        self.c2 = [Convolver(shape, k, self.device) for k in k2]
        self.avg = first_iteration_average(self.views)
        # the library and the numpy oracle start from psi = (float) avg
        self.psi = torch.full(shape, float(np.float32(self.avg)), **dd)
        self.stats = []
        self.iteration = 0

    def run_view(self, v):
        blurred = self.c1[v](self.psi, O.MIRROR)
        img = self.views[v]
        q = torch.where(img > 0, img / blurred, torch.ones_like(img))  # computeQuotient (:494-546)
        integral = self.c2[v](q, O.VALUE, 1.0)
        # computeFinalValues / computeNextValue / tikhonov (MVDeconvolution.java:603-726)
        last = self.psi
        value = last * integral
        if self.lam > 0:
            adj = torch.where(value > 0, (torch.sqrt(1.0 + 2.0 * self.lam * value) - 1.0) / self.lam,
                              torch.full_like(value, float(O.MIN_VALUE)))
        else:
            adj = torch.where(value > 0, value, torch.full_like(value, float(O.MIN_VALUE)))
        nxt = torch.where(torch.isnan(adj), torch.full_like(adj, float(O.MIN_VALUE)),
                          torch.clamp(adj, min=float(O.MIN_VALUE)))
        new = last + (nxt - last) * self.weights[v]
        change = (new - last).abs()
        self.psi = new
        s, m = float(change.sum().item()), float(change.max().item())
        self.stats.append((self.iteration, v, s, m))
        return s, m

    def run_iteration(self):
        for v in range(len(self.views)):
            self.run_view(v)
        self.iteration += 1

    def run(self, iterations):
        for _ in range(iterations):
            self.run_iteration()
        return self.psi

    def masked_psi(self) -> torch.Tensor:
        """psi := 0 where no view has data (MVDeconvolution.java:201-208)."""
        any_pos = torch.zeros_like(self.psi, dtype=torch.bool)
        for v in self.views:
            any_pos |= v > 0
        return torch.where(any_pos, self.psi, torch.zeros_like(self.psi))


def errors(got, want: torch.Tensor) -> dict:
    """Relative L2 and max-abs error of a float32 result against the float64 one (on want's
    device), plus the max-abs error relative to the largest value."""
    g = torch.as_tensor(np.asarray(got, dtype=np.float32) if not torch.is_tensor(got) else got)
    g = g.to(device=want.device, dtype=torch.float64)
    d = g - want
    norm = float(torch.linalg.vector_norm(want).item())
    mx = float(want.abs().max().item())
    max_abs = float(d.abs().max().item())
    return {"rel_l2": float(torch.linalg.vector_norm(d).item()) / max(norm, 1e-300), "max_abs": max_abs,
            "max_abs_rel": max_abs / max(mx, 1e-300)}


def poisson_nll(psi, views, weights, psfs, device="cuda") -> float:
    """``mvdecon_oracle.poisson_nll`` in float64 on ``device``: sum over views and voxels with
    img > 0 of w (f - img log f), f = ext(psi) (*) P (mirror-single extension)."""
    dd = dict(device=torch.device(device), dtype=torch.float64)
    p = torch.as_tensor(np.asarray(psi, dtype=np.float64)).to(**dd)
    total = 0.0
    for img, w, k in zip(views, weights, psfs):
        f = Convolver(p.shape, np.asarray(k, dtype=np.float64), dd["device"])(p, O.MIRROR)
        im = torch.as_tensor(np.asarray(img, dtype=np.float32)).to(**dd)
        wt = torch.as_tensor(np.asarray(w, dtype=np.float32)).to(**dd)
        m = im > 0
        total += float((wt[m] * (f[m] - im[m] * torch.log(f[m]))).sum().item())
    return total
