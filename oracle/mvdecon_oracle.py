"""CPU oracle for the multiview Bayesian deconvolution path.  TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use this
module, to check results or as the timed CPU restatement; the library never calls it.

PARITY UNPINNED.  fiji/SPIM_Registration ships no tests, golden vectors or fixtures for this
path, and the reference is Java (Maven, imglib2) with no JDK available to run it, so this file
is a restatement of the reference's algorithm, anchored on known-answer tests
(``tests/test_oracle.py``) rather than on outputs of the reference itself.

Two arithmetic modes:

* ``"f64"``  -- every step in float64 (the FP64 oracle against which relative L2 is stated);
* ``"f32"``  -- the Java ``float`` semantics of the reference loops (float multiplies and
  divides, Tikhonov in double then rounded, FP64 statistics) with float32 FFTs.

Citations are paths under the reference's ``src/main/java``.

The CPU FFT convolution is ``net.imglib2.algorithm.fft2.FFTConvolution`` (imglib2-algorithm,
version managed by ``org.scijava:pom-scijava:34.1.0``, imglib2 6.1.0; not vendored).  Its
published behaviour, restated here: the image is extended by its out-of-bounds strategy
(mirror-single unless the caller passes another), the kernel is zero-extended with its centre
at ``size // 2``, the product of the spectra is inverted (``computeComplexConjugate=false``:
true convolution) and the result is cropped to the image interval.  With the padded size at
least ``image + kernel - 1`` this equals the linear convolution of the extended image, which is
what ``conv_extended`` computes.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.fft

MIN_VALUE = np.float32(1e-4)  # MVDeconvolution.java:70

OPTIMIZATION_II, OPTIMIZATION_I, EFFICIENT_BAYESIAN, INDEPENDENT = 0, 1, 2, 3  # MVDeconFFT.java:49

MIRROR, VALUE = 0, 1  # out-of-bounds strategies used on the path


def _workers():
    import os

    return os.cpu_count() or 1


# --------------------------------------------------------------------------------------------
# helpers restated from the reference
# --------------------------------------------------------------------------------------------
def divide_into_portions(size: int, n: int):
    """FusionHelper.divideIntoPortions (spim/process/fusion/FusionHelper.java:257-280)."""
    chunk, mod = divmod(size, n)
    out = []
    for p in range(n):
        start = p * chunk
        loop = chunk + mod if p == n - 1 else chunk
        out.append((start, loop))
    return out


def sum_img(k: np.ndarray, quirk_threads: int | None = None) -> float:
    """AdjustInput.sumImg (AdjustInput.java:70-121), FP64.

    With ``quirk_threads`` set, portion 0 of ``2 * threads`` portions is added twice, as the
    reference does (``sum.add(sums[0])`` before the loop over all portions, :114-118).
    """
    flat = k.astype(np.float64).ravel()
    total = math.fsum(flat)
    if quirk_threads:
        start, loop = divide_into_portions(flat.size, 2 * quirk_threads)[0]
        total += math.fsum(flat[start:start + loop])
    return total


def norm_img(k: np.ndarray, quirk_threads: int | None = None, mode: str = "f64") -> np.ndarray:
    """AdjustInput.normImg (AdjustInput.java:50-56): t = (float)((double)t / sum)."""
    s = sum_img(k, quirk_threads)
    out = k.astype(np.float64) / s
    return out.astype(np.float32) if mode == "f32" else out


def mirror(k: np.ndarray) -> np.ndarray:
    """Mirror.mirror applied along every dimension (MVDeconFFT.computeInvertedKernel :336-344).

    Mirror.java:52-129 swaps position p with n-1-p for every p <= n/2.  For odd n that is a
    flip; for even n the pair (n/2-1, n/2) is swapped twice and so stays in place.
    """
    out = np.array(k, copy=True)
    for axis in range(out.ndim):
        n = out.shape[axis]
        out = np.flip(out, axis=axis)
        if n % 2 == 0 and n >= 2:
            idx = [slice(None)] * out.ndim
            a, b = list(idx), list(idx)
            a[axis], b[axis] = n // 2 - 1, n // 2
            ta, tb = out[tuple(a)].copy(), out[tuple(b)].copy()
            out[tuple(a)], out[tuple(b)] = tb, ta
    return np.ascontiguousarray(out)


def mirror_single_index(idx: np.ndarray, n: int) -> np.ndarray:
    """imglib2 OutOfBoundsMirrorSingleBoundary index map: -1 -> 1, n -> n-2, period 2n-2."""
    if n == 1:
        return np.zeros_like(idx)
    period = 2 * n - 2
    m = np.mod(idx, period)
    return np.where(m < n, m, period - m)


def extend(img: np.ndarray, pad_lo, pad_hi, mode: int, value: float = 0.0) -> np.ndarray:
    """Views.extendMirrorSingle / Views.extendValue restricted to a padded interval."""
    if mode == MIRROR:
        ix = [mirror_single_index(np.arange(-pad_lo[d], img.shape[d] + pad_hi[d]), img.shape[d])
              for d in range(img.ndim)]
        return img[np.ix_(*ix)]
    out = np.full([img.shape[d] + pad_lo[d] + pad_hi[d] for d in range(img.ndim)], value,
                  dtype=img.dtype)
    out[tuple(slice(pad_lo[d], pad_lo[d] + img.shape[d]) for d in range(img.ndim))] = img
    return out


def conv_extended(img: np.ndarray, kernel: np.ndarray, mode: int = MIRROR, value: float = 0.0,
                  arith: str = "f64") -> np.ndarray:
    """Linear convolution of the extended image with the centred kernel, cropped to the image.

    out[x] = sum_j kernel[j] * ext(img)[x - (j - k//2)]   (true convolution)

    This is what FFTConvolution computes on the image interval (MVDeconFFT.java:384-560,
    MVDeconFFTThreads.java:39-70) and what the blocked path computes on each block's effective
    region (Block.java:134-379).
    """
    dt = np.float64 if arith == "f64" else np.float32
    h = [s // 2 for s in kernel.shape]
    hi = [s - 1 - s // 2 for s in kernel.shape]
    # out[x] needs ext(img)[x - (j - h)] for j in [0, k): offsets -(k-1-h) .. +h
    ext = extend(img.astype(dt), hi, h, mode, value)
    shape = [ext.shape[d] + kernel.shape[d] - 1 for d in range(img.ndim)]
    fshape = [scipy.fft.next_fast_len(s, real=True) for s in shape]
    fa = scipy.fft.rfftn(ext, fshape, workers=_workers())
    fb = scipy.fft.rfftn(kernel.astype(dt), fshape, workers=_workers())
    full = scipy.fft.irfftn(fa * fb, fshape, workers=_workers())
    sl = tuple(slice(kernel.shape[d] - 1, kernel.shape[d] - 1 + img.shape[d]) for d in range(img.ndim))
    return np.ascontiguousarray(full[sl]).astype(dt)


def conv_direct(img: np.ndarray, kernel: np.ndarray, mode: int = MIRROR, value: float = 0.0) -> np.ndarray:
    """Spatial-domain restatement of conv_extended (FP64), for known-answer tests."""
    img = img.astype(np.float64)
    k = kernel.astype(np.float64)
    h = [s // 2 for s in k.shape]
    hi = [s - 1 - s // 2 for s in k.shape]
    ext = extend(img, hi, h, mode, value)
    out = np.zeros(img.shape, dtype=np.float64)
    kz, ky, kx = k.shape
    nz, ny, nx = img.shape
    for jz in range(kz):
        for jy in range(ky):
            for jx in range(kx):
                # ext index of img position x - (j - h) is x - (j - h) + hi
                oz, oy, ox = hi[0] - (jz - h[0]), hi[1] - (jy - h[1]), hi[2] - (jx - h[2])
                out += k[jz, jy, jx] * ext[oz:oz + nz, oy:oy + ny, ox:ox + nx]
    return out


# --------------------------------------------------------------------------------------------
# blocking (BlockGeneratorFixedSizePrecise + Block copy/paste)
# --------------------------------------------------------------------------------------------
def divide_into_blocks(img_xyz, kernel_xyz, block_xyz):
    """BlockGeneratorFixedSizePrecise.divideIntoBlocks (BlockGeneratorFixedSizePrecise.java:46-122).

    Returns a list of dicts with ``offset``, ``eff_offset``, ``eff_size``, ``eff_local`` in
    (x, y, z) order; blocks are enumerated x fastest.
    """
    n = len(img_xyz)
    eff = [block_xyz[d] - kernel_xyz[d] + 1 for d in range(n)]
    if any(e <= 0 for e in eff):
        raise ValueError("block smaller than kernel")
    local = [kernel_xyz[d] // 2 for d in range(n)]
    nblk = [img_xyz[d] // eff[d] + (1 if img_xyz[d] % eff[d] else 0) for d in range(n)]
    blocks = []
    for bz in range(nblk[2]):
        for by in range(nblk[1]):
            for bx in range(nblk[0]):
                cur = (bx, by, bz)
                eo = [cur[d] * eff[d] for d in range(n)]
                es = [min(eff[d], img_xyz[d] - eo[d]) for d in range(n)]
                off = [eo[d] - kernel_xyz[d] // 2 for d in range(n)]
                blocks.append(dict(offset=off, eff_offset=eo, eff_size=es, eff_local=local))
    return blocks


def convolve_blocked(img: np.ndarray, kernel: np.ndarray, block_xyz, mode: int, value: float = 0.0,
                     arith: str = "f64") -> np.ndarray:
    """MVDeconFFT.convolve1/convolve2 with blocks (MVDeconFFT.java:386-410, 481-503).

    Each block is copied from the extended image (Block.copyBlock :134-173), convolved with its
    own mirror-single extension (MVDeconFFTThreads.java:45-48) and its effective region pasted
    (Block.pasteBlock :175-215).
    """
    nz, ny, nx = img.shape
    kz, ky, kx = kernel.shape
    blocks = divide_into_blocks((nx, ny, nz), (kx, ky, kz), block_xyz)
    out = np.zeros(img.shape, dtype=np.float64 if arith == "f64" else np.float32)
    bx, by, bz = block_xyz
    for b in blocks:
        ox, oy, oz = b["offset"]
        pad = [max(0, -oz), max(0, -oy), max(0, -ox)]
        hi = [max(0, oz + bz - nz), max(0, oy + by - ny), max(0, ox + bx - nx)]
        ext = extend(img, pad, hi, mode, value)
        blk = ext[oz + pad[0]:oz + pad[0] + bz, oy + pad[1]:oy + pad[1] + by, ox + pad[2]:ox + pad[2] + bx]
        conv = conv_extended(blk, kernel, MIRROR, 0.0, arith)
        ex, ey, ez = b["eff_offset"]
        sx, sy, sz = b["eff_size"]
        lx, ly, lz = b["eff_local"]
        out[ez:ez + sz, ey:ey + sy, ex:ex + sx] = conv[lz:lz + sz, ly:ly + sy, lx:lx + sx]
    return out


# --------------------------------------------------------------------------------------------
# kernel preparation (MVDeconFFT.init)
# --------------------------------------------------------------------------------------------
def _pow_float(k: np.ndarray, power: int) -> np.ndarray:
    """MVDeconFFT.pow (:346-354): repeated float multiplication."""
    out = k.copy()
    for _ in range(1, power):
        out = (out * k).astype(k.dtype)
    return out


def prepare_kernels(psfs, psftype: int, quirk_threads: int | None = None, arith: str = "f64"):
    """MVDeconFFT.init (MVDeconFFT.java:183-324) for every view.

    Returns (kernel1, kernel2) lists.  kernel1 = normImg(psf); kernel2 by PSFTYPE:
    INDEPENDENT (or one view): mirror(P_v); EFFICIENT_BAYESIAN:
    norm(mirror(P_v) * prod_{w != v} crop(crop(mirror(P_v) (*) P_w) (*) mirror(P_w)));
    OPTIMIZATION_I: mirror(norm(P_v * prod_{w != v} crop(P_v (*) mirror(P_w))));
    OPTIMIZATION_II: mirror(norm(P_v ** V)).  (*) is FFTConvolution with zero extension,
    cropped to P_v's interval.
    """
    k1 = [norm_img(p, quirk_threads, arith) for p in psfs]
    nv = len(k1)
    k2 = []
    for v in range(nv):
        if nv == 1 or psftype == INDEPENDENT:
            k2.append(mirror(k1[v]))
        elif psftype == EFFICIENT_BAYESIAN:
            tmp = mirror(k1[v])
            for w in range(nv):
                if w == v:
                    continue
                out = conv_extended(mirror(k1[v]), k1[w], VALUE, 0.0, arith)
                out = conv_extended(out, mirror(k1[w]), VALUE, 0.0, arith)
                tmp = tmp * out
            k2.append(norm_img(tmp, quirk_threads, arith))
        elif psftype == OPTIMIZATION_I:
            tmp = k1[v].copy()
            for w in range(nv):
                if w == v:
                    continue
                out = conv_extended(k1[v], mirror(k1[w]), VALUE, 0.0, arith)
                tmp = tmp * out
            k2.append(mirror(norm_img(tmp, quirk_threads, arith)))
        else:
            e = _pow_float(k1[v].astype(np.float32) if arith == "f32" else k1[v], nv)
            k2.append(mirror(norm_img(e, quirk_threads, arith)))
    return k1, k2


# --------------------------------------------------------------------------------------------
# first iteration, quotient, update (MVDeconvolution)
# --------------------------------------------------------------------------------------------
def first_iteration(views):
    """FirstIteration.call + MVDeconvolution.fuseFirstIteration (FirstIteration.java:84-154,
    MVDeconvolution.java:213-256, :133-147).  Returns (avg, count_image)."""
    s = np.zeros(views[0].shape, dtype=np.float64)
    c = np.zeros(views[0].shape, dtype=np.int32)
    for v in views:
        pos = v > 0
        s += np.where(pos, v.astype(np.float64), 0.0)
        c += pos
    has = c > 0
    mean = np.where(has, s / np.maximum(c, 1), 0.0)
    count = int(has.sum())
    avg = math.fsum(mean[has].ravel()) / count if count else float("nan")
    if math.isnan(avg):
        avg = 0.5  # MVDeconvolution.java:138-142
    return avg, c


def compute_quotient(blurred: np.ndarray, img: np.ndarray, arith: str = "f64") -> np.ndarray:
    """MVDeconvolution.computeQuotient (:494-546): img > 0 ? img / blurred : 1."""
    dt = np.float64 if arith == "f64" else np.float32
    with np.errstate(divide="ignore", invalid="ignore"):
        q = img.astype(dt) / blurred.astype(dt)
    return np.where(img > 0, q, dt(1)).astype(dt)


def compute_final_values(psi, integral, weight, lam: float, arith: str = "f64"):
    """computeFinalValues / computeNextValue / tikhonov (MVDeconvolution.java:603-726).

    Returns (new_psi, sum_change, max_change); statistics in FP64 as the reference does.
    """
    if arith == "f32":
        last = psi.astype(np.float32)
        value = (last * integral.astype(np.float32)).astype(np.float32)
        with np.errstate(invalid="ignore", over="ignore"):
            if lam > 0:
                vd = value.astype(np.float64)
                tik = ((np.sqrt(1.0 + 2.0 * lam * vd) - 1.0) / lam).astype(np.float32)
                adj = np.where(value > 0, tik, MIN_VALUE).astype(np.float32)
            else:
                adj = np.where(value > 0, value, MIN_VALUE).astype(np.float32)
            nxt = np.where(np.isnan(adj), MIN_VALUE, np.maximum(MIN_VALUE, adj)).astype(np.float32)
            diff = (nxt - last).astype(np.float32)
            new = (last + (diff * weight.astype(np.float32)).astype(np.float32)).astype(np.float32)
        change = np.abs(new - last).astype(np.float32).astype(np.float64)
    else:
        last = psi.astype(np.float64)
        value = last * integral.astype(np.float64)
        with np.errstate(invalid="ignore", over="ignore"):
            if lam > 0:
                tik = (np.sqrt(1.0 + 2.0 * lam * value) - 1.0) / lam
                adj = np.where(value > 0, tik, float(MIN_VALUE))
            else:
                adj = np.where(value > 0, value, float(MIN_VALUE))
            nxt = np.where(np.isnan(adj), float(MIN_VALUE), np.maximum(float(MIN_VALUE), adj))
            new = last + (nxt - last) * weight.astype(np.float64)
        change = np.abs(new - last)
    return new, float(change.sum()), float(change.max()) if change.size else -1.0


class Deconvolution:
    """MVDeconvolution (MVDeconvolution.java:94-211, 354-465) restated over numpy arrays.

    ``views``, ``weights`` are [z,y,x] arrays; ``psfs`` odd-sized [kz,ky,kx] arrays.
    ``block`` = (bx, by, bz) runs the blocked convolutions of MVDeconFFT; None = one image.
    """

    def __init__(self, views, weights, psfs, psftype, lam, arith="f64", block=None,
                 quirk_threads=None, psi0=None):
        self.arith = arith
        self.dt = np.float64 if arith == "f64" else np.float32
        self.views = [np.asarray(v, dtype=np.float32) for v in views]
        self.weights = [np.asarray(w, dtype=np.float32) for w in weights]
        self.lam = float(lam)
        self.block = block
        self.k1, self.k2 = prepare_kernels(psfs, psftype, quirk_threads, arith)
        if psi0 is None:
            avg, _ = first_iteration(self.views)
            self.avg = avg
            self.psi = np.full(self.views[0].shape, np.float32(avg), dtype=self.dt)
        else:
            self.psi = np.asarray(psi0, dtype=self.dt).copy()
        self.stats = []
        self.iteration = 0

    def _conv(self, img, kernel, mode, value):
        if self.block is None:
            return conv_extended(img, kernel, mode, value, self.arith)
        return convolve_blocked(img, kernel, self.block, mode, value, self.arith)

    def run_view(self, v):
        blurred = self._conv(self.psi, self.k1[v], MIRROR, 0.0)
        q = compute_quotient(blurred, self.views[v], self.arith)
        integral = self._conv(q, self.k2[v], VALUE, 1.0)
        self.psi, s, m = compute_final_values(self.psi, integral, self.weights[v], self.lam, self.arith)
        self.psi = self.psi.astype(self.dt)
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

    def masked_psi(self):
        """Masking of never-updated voxels (MVDeconvolution.java:201-208)."""
        _, count = first_iteration(self.views)
        return np.where(count == 0, 0, self.psi).astype(self.dt)


def deconvolve(problem, iterations=None, arith="f64", block="problem", quirk_threads=None,
               mask=True):
    """Run a synthetic ``Problem`` through the restated reference loop."""
    blk = problem.block if block == "problem" else block
    d = Deconvolution(problem.views, problem.weights, problem.psfs, problem.psftype, problem.lam,
                      arith, blk, quirk_threads)
    d.run(problem.iterations if iterations is None else iterations)
    return (d.masked_psi() if mask else d.psi), d


# --------------------------------------------------------------------------------------------
# image-formation model and its gradients (checker of the forward/backward pair)
# --------------------------------------------------------------------------------------------
def poisson_nll(psi, views, weights, psfs):
    """NLL(psi, P) = sum_v sum_{x: img_v > 0} w_v [f_v - img_v log f_v],  f_v = ext(psi) (*) P_v.

    ext is the mirror-single extension of the first convolution of an iteration
    (MVDeconFFTThreads.java:44,78); the PSFs are used as given; FP64.
    """
    total = 0.0
    for img, w, p in zip(views, weights, psfs):
        f = conv_extended(np.asarray(psi, dtype=np.float64), p, MIRROR, 0.0, "f64")
        m = img > 0
        total += math.fsum((w[m].astype(np.float64) * (f[m] - img[m].astype(np.float64) * np.log(f[m]))).ravel())
    return total


def fold_mirror(c: np.ndarray, n_shape, h):
    """Adjoint of the mirror-single extension: c lives on [-h, n+h) per axis; every extended
    position adds into the voxel it mirrors."""
    out = c
    for axis in range(3):
        n, hh = n_shape[axis], h[axis]
        idx = mirror_single_index(np.arange(-hh, n + hh), n)
        moved = np.moveaxis(out, axis, 0)
        acc = np.zeros((n,) + moved.shape[1:], dtype=np.float64)
        np.add.at(acc, idx, moved)
        out = np.moveaxis(acc, 0, axis)
    return out


def poisson_nll_grad(psi, views, weights, psfs):
    """Analytic gradients of poisson_nll w.r.t. psi and every PSF voxel (FP64).

    r_v = w_v (1 - img_v / f_v) on img_v > 0 (else 0);
    dNLL/dpsi   = sum_v fold( r_v (zero-extended) (*) mirror(P_v) on [-h, n+h) );
    dNLL/dP_v(j) = sum_x r_v(x) ext(psi)(x - (j - k/2)).
    """
    psi = np.asarray(psi, dtype=np.float64)
    g_psi = np.zeros_like(psi)
    g_psf = []
    for img, w, p in zip(views, weights, psfs):
        p = np.asarray(p, dtype=np.float64)
        f = conv_extended(psi, p, MIRROR, 0.0, "f64")
        m = img > 0
        r = np.where(m, w.astype(np.float64) * (1.0 - img.astype(np.float64) / np.where(m, f, 1.0)), 0.0)
        h = [s // 2 for s in p.shape]
        r_ext = extend(r, h, h, VALUE, 0.0)
        c = conv_extended(r_ext, mirror(p), VALUE, 0.0, "f64")
        g_psi += fold_mirror(c, psi.shape, h)
        hi = [s - 1 - s // 2 for s in p.shape]
        pe = extend(psi, h, hi, MIRROR)  # pe[u + h] = ext(psi)(u), u in [-h, n + hi)
        nz, ny, nx = psi.shape
        g = np.zeros(p.shape)
        for jz in range(p.shape[0]):
            for jy in range(p.shape[1]):
                for jx in range(p.shape[2]):
                    # ext(psi)(x - (j - h)) = pe[x - j + 2h]
                    oz, oy, ox = 2 * h[0] - jz, 2 * h[1] - jy, 2 * h[2] - jx
                    g[jz, jy, jx] = np.sum(r * pe[oz:oz + nz, oy:oy + ny, ox:ox + nx])
        g_psf.append(g)
    return g_psi, g_psf


# --------------------------------------------------------------------------------------------
# input preparation: views in the fused frame, blending weights, VIRTUAL normalisation
# --------------------------------------------------------------------------------------------
def _inverse_affine(affine_rows):
    a = np.asarray(affine_rows, dtype=np.float64).reshape(3, 4)
    r_inv = np.linalg.inv(a[:, :3])
    return r_inv, -r_inv @ a[:, 3]


def _view_positions(affine_rows, offset_xyz, out_shape_zyx):
    nz, ny, nx = out_shape_zyx
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    s = np.stack([x + offset_xyz[0], y + offset_xyz[1], z + offset_xyz[2]], axis=-1).astype(np.float64)
    r_inv, t = _inverse_affine(affine_rows)
    return s @ r_inv.T + t  # (..., 3) view coordinates (x, y, z)


def transform_input(view, affine_rows, offset_xyz, out_shape_zyx):
    """TransformInput.loop (TransformInput.java:90-116), FP64: trilinear interpolation of the
    mirror-single extended view at affine^-1(position); max(minValue, .) inside the view, 0
    outside (FusionHelper.intersects, FusionHelper.java:75-81)."""
    v = np.asarray(view, dtype=np.float64)
    sz, sy, sx = v.shape
    t = _view_positions(affine_rows, offset_xyz, out_shape_zyx)
    f = np.floor(t)
    a = t - f
    i0 = f.astype(np.int64)
    out = np.zeros(t.shape[:-1])
    for c in range(8):
        bx, by, bz = c & 1, (c >> 1) & 1, (c >> 2) & 1
        xi = mirror_single_index(i0[..., 0] + bx, sx)
        yi = mirror_single_index(i0[..., 1] + by, sy)
        zi = mirror_single_index(i0[..., 2] + bz, sz)
        w = (a[..., 0] if bx else 1 - a[..., 0]) * (a[..., 1] if by else 1 - a[..., 1]) * (a[..., 2] if bz else 1 - a[..., 2])
        out += w * v[zi, yi, xi]
    inside = (t[..., 0] >= 0) & (t[..., 1] >= 0) & (t[..., 2] >= 0) & (t[..., 0] < sx) & (t[..., 1] < sy) & (t[..., 2] < sz)
    return np.where(inside, np.maximum(float(MIN_VALUE), out), 0.0)


def _blend_lut():
    """The lookup table as BlendingRealRandomAccess's static block fills it (:47-53): d steps by
    0.001 in double from 0 while d <= 1.0001, and entry round(d * 1000) holds the value at the
    accumulated d (which drifts from k / 1000 in the last bits)."""
    lut = np.zeros(1001)
    d = 0.0
    while d <= 1.0001:
        lut[int(math.floor(d * 1000.0 + 0.5))] = (math.cos((1 - d) * math.pi) + 1) / 2
        d = d + 0.001
    return lut


_BLEND_LUT = _blend_lut()


def transform_weights(view_shape_zyx, affine_rows, offset_xyz, out_shape_zyx, border_xyz, blending_xyz):
    """TransformWeights + BlendingRealRandomAccess.computeWeight (BlendingRealRandomAccess.java:
    44-121): the cosine blending weight at affine^-1(position) over the view interval, with
    the 1001-entry lookup table (index round(d * 1000))."""
    sz, sy, sx = view_shape_zyx
    t = _view_positions(affine_rows, offset_xyz, out_shape_zyx).astype(np.float32)
    dm1 = (sx - 1, sy - 1, sz - 1)
    w = np.ones(t.shape[:-1], dtype=np.float32)
    zero = np.zeros(t.shape[:-1], dtype=bool)
    for d in range(3):
        l = t[..., d]
        dist = np.maximum(np.float32(0), np.minimum(l - np.float32(border_xyz[d]),
                                                    np.float32(dm1[d]) - l - np.float32(border_xyz[d])))
        zero |= dist == 0
        rel = (dist / np.float32(blending_xyz[d])).astype(np.float32)
        idx = np.floor(rel.astype(np.float64) * 1000.0 + 0.5).astype(np.int64)
        lut = _BLEND_LUT[np.clip(idx, 0, 1000)]
        w = np.where(rel < 1, (w.astype(np.float64) * lut).astype(np.float32), w)
    return np.where(zero, np.float32(0), w).astype(np.float32)


def normalize_weights_virtual(weights, osem=1.0):
    """VIRTUAL weights (WeightNormalizer.java:73-253, NormalizingRandomAccess.java:57-66):
    w_v / (sum > 1 ? (float)sum : 1), then min(1, w * osem)."""
    s = np.zeros(weights[0].shape, dtype=np.float64)
    for w in weights:
        s += w.astype(np.float64)
    norm = np.where(s > 1, s.astype(np.float32), np.float32(1)).astype(np.float64)
    return [np.minimum(1.0, w.astype(np.float64) / norm * osem).astype(np.float32) for w in weights]


def normalize_weights_precomputed(weights, osem=1.0):
    """PRECOMPUTED weights (WeightNormalizer.ApplyDirectly, WeightNormalizer.java:132-185, then
    ProcessForDeconvolution.adjustForOSEM, :376-383): (float)(w_v / sum) with no guard on the
    sum (NaN where every view has weight 0), then Math.min(1, w * (float)osem) in float, NaN
    kept (Math.min propagates NaN)."""
    s = np.zeros(weights[0].shape, dtype=np.float64)
    for w in weights:
        s += w.astype(np.float64)
    out = []
    with np.errstate(invalid="ignore", divide="ignore"):
        for w in weights:
            x = (w.astype(np.float64) / s).astype(np.float32)
            y = x * np.float32(osem)
            out.append(np.where(np.isnan(y), y, np.minimum(np.float32(1), y)).astype(np.float32))
    return out


def weight_overlap(weights, num_portions):
    """WeightNormalizer's overlap statistics (WeightNormalizer.java:94-106, 187-252): the minimum
    per-voxel count of views with weight > 0, and the mean over the portions of
    divideIntoPortions(n, num_portions) of each portion's mean count."""
    count = np.zeros(weights[0].size, dtype=np.int64)
    for w in weights:
        count += (w.ravel() > 0)
    avg = 0.0
    for start, loop in divide_into_portions(count.size, num_portions):
        avg += float(count[start:start + loop].sum()) / loop
    return int(count.min()), avg / num_portions


# --------------------------------------------------------------------------------------------
# separable convolution (the difference-of-Gaussian detector's native library)
# --------------------------------------------------------------------------------------------
SEP_ZERO, SEP_VALUE, SEP_EXTEND = 0, 1, 2


def separable_convolve(image, kernels_xyz, oob, value=0.0):
    """CUDASeparableConvolution.convolve_K (CUDASeparableConvolution.java:34-46), restated from the
    behaviour the interface documents (the native SeparableConvolutionCUDALib is an external
    project, not vendored): in place along x, then y, then z (a None kernel skips its axis);
    out[x] = sum_{j=-R..R} in[x + j] k[R - j]; each pass extends its own input (0 zero,
    1 value, 2 border pixel) and is stored as float32.  Accumulates in FP64."""
    out = np.asarray(image, dtype=np.float32)
    for axis_xyz, k in enumerate(kernels_xyz):
        if k is None:
            continue
        ax = out.ndim - 1 - axis_xyz
        if ax < 0:
            continue
        k = np.asarray(k, dtype=np.float64)
        R = len(k) // 2
        pad = [(0, 0)] * out.ndim
        pad[ax] = (R, R)
        if oob == SEP_EXTEND:
            p = np.pad(out.astype(np.float64), pad, mode="edge")
        else:
            cval = float(np.float32(value)) if oob == SEP_VALUE else 0.0
            p = np.pad(out.astype(np.float64), pad, mode="constant", constant_values=cval)
        n = out.shape[ax]
        acc = np.zeros(out.shape, dtype=np.float64)
        for m in range(2 * R + 1):
            sl = [slice(None)] * out.ndim
            sl[ax] = slice(m, m + n)
            acc += p[tuple(sl)] * k[2 * R - m]
        out = acc.astype(np.float32)
    return out


# --------------------------------------------------------------------------------------------
# PSF pipeline (ExtractPSF)
# --------------------------------------------------------------------------------------------
def _trilinear(v, t, periodic):
    """Trilinear interpolation of v [z, y, x] at positions t (..., 3) = (x, y, z), FP64; the
    volume is extended periodically or with zeros."""
    sz, sy, sx = v.shape
    f = np.floor(t)
    a = t - f
    i0 = f.astype(np.int64)
    out = np.zeros(t.shape[:-1])
    for c in range(8):
        b = [(c >> k) & 1 for k in range(3)]
        idx = [i0[..., k] + b[k] for k in range(3)]
        w = np.ones(t.shape[:-1])
        for k in range(3):
            w = w * (a[..., k] if b[k] else 1 - a[..., k])
        if periodic:
            val = v[np.mod(idx[2], sz), np.mod(idx[1], sy), np.mod(idx[0], sx)]
        else:
            ok = (idx[0] >= 0) & (idx[1] >= 0) & (idx[2] >= 0) & (idx[0] < sx) & (idx[1] < sy) & (idx[2] < sz)
            val = np.where(ok, v[np.clip(idx[2], 0, sz - 1), np.clip(idx[1], 0, sy - 1), np.clip(idx[0], 0, sx - 1)], 0)
        out += w * val
    return out


def extract_psf_local(img, locations_xyz, psf_dims_xyz, normalize=False):
    """ExtractPSF.extractPSFLocal (ExtractPSF.java:374-415): the sum over the bead locations of the
    periodically extended image interpolated at p - size / 2 + location; with ``normalize``,
    ExtractPSF.normalize (:298-316), (v - min) / (max - min)."""
    v = np.asarray(img, dtype=np.float64)
    px, py, pz = psf_dims_xyz
    z, y, x = np.meshgrid(np.arange(pz), np.arange(py), np.arange(px), indexing="ij")
    base = np.stack([x - px // 2, y - py // 2, z - pz // 2], axis=-1).astype(np.float64)
    psf = np.zeros((pz, py, px))
    for loc in locations_xyz:
        psf += _trilinear(v, base + np.asarray(loc, dtype=np.float64), periodic=True)
    if normalize:
        lo, hi = psf.min(), psf.max()
        psf = (psf - lo) / (hi - lo)
    return psf


def transformed_psf_size(psf_dims_xyz, model_rows):
    """ExtractPSF.transformPSF (:325-372): odd output size and offset."""
    a = np.asarray(model_rows, dtype=np.float64).reshape(3, 4)
    corners = np.array([[(c & 1) * (psf_dims_xyz[0] - 1), ((c >> 1) & 1) * (psf_dims_xyz[1] - 1),
                         ((c >> 2) & 1) * (psf_dims_xyz[2] - 1)] for c in range(8)], dtype=np.float64)
    t = corners @ a[:, :3].T + a[:, 3]
    size = t.max(axis=0) - t.min(axis=0)
    ns = [int(s) + 1 for s in size]
    ns = [n + 1 if n % 2 == 0 else n for n in ns]
    ctr = np.array([d // 2 for d in psf_dims_xyz], dtype=np.float64)
    tc = a[:, :3] @ ctr + a[:, 3]
    return ns, [tc[d] - ns[d] // 2 for d in range(3)]


def transform_psf(psf, model_rows, out_dims_xyz, offset_xyz):
    """ExtractPSF.transform (:417-464): out[p] = psf(model^-1 (p + offset)), trilinear, zero outside."""
    a = np.asarray(model_rows, dtype=np.float64).reshape(3, 4)
    r_inv = np.linalg.inv(a[:, :3])
    nx, ny, nz = out_dims_xyz
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    p = np.stack([x + offset_xyz[0], y + offset_xyz[1], z + offset_xyz[2]], axis=-1).astype(np.float64)
    t = (p - a[:, 3]) @ r_inv.T
    return _trilinear(np.asarray(psf, dtype=np.float64), t, periodic=False)
