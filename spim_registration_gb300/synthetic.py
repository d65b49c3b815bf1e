"""Seeded synthetic multiview inputs for the deconvolution path.

The Java host prepares the per-view inputs before ``MVDeconvolution`` runs: every view
resampled into the fused bounding box (``TransformInput.java:90-116``), its blending weight
(``BlendingRealRandomAccess.java:44-121``) normalised across views
(``WeightNormalizer.java:73-253``, ``NormalizingRandomAccess.java:57-66``) and the PSF
transformed into the fused frame (``ExtractPSF.java:325-364``).  No public dataset exists for
this path, so this module builds those inputs from seeded synthetic ground truth:

* ground truth: 3D Gaussian blobs on a constant background;
* PSF: an anisotropic Gaussian, rotated about the y axis per view, odd sizes with the centre
  voxel at ``size // 2`` (the size rule of ``ExtractPSF.transformPSF``);
* view image: ground truth blurred by that view's PSF (mirror-single border), Poisson noise,
  clamped to ``minValue`` so that ``img > 0`` marks data (``TransformInput.java:103-110``);
* weights: cosine blending in the view's rotated frame, then the VIRTUAL normalisation
  ``w_v / (sum_w > 1 ? sum_w : 1)`` and ``min(1, w * osem)``.

Arrays are numpy ``float32`` in ``[z, y, x]`` order (x fastest, the ``ArrayImg`` layout);
sizes in the public API are ``(x, y, z)`` like the Java ``long[]`` dimensions.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

MIN_VALUE = np.float32(1e-4)  # MVDeconvolution.minValue (MVDeconvolution.java:70)

# PSFTYPE ordinals (MVDeconFFT.java:49)
OPTIMIZATION_II, OPTIMIZATION_I, EFFICIENT_BAYESIAN, INDEPENDENT = 0, 1, 2, 3
PSFTYPE_NAMES = {
    "OPTIMIZATION_II": OPTIMIZATION_II,
    "OPTIMIZATION_I": OPTIMIZATION_I,
    "EFFICIENT_BAYESIAN": EFFICIENT_BAYESIAN,
    "INDEPENDENT": INDEPENDENT,
}


@dataclasses.dataclass
class Problem:
    """One deconvolution job: everything ``MVDeconvolution``'s constructor receives."""

    name: str
    views: list  # list of float32 [z,y,x]
    weights: list  # list of float32 [z,y,x]
    psfs: list  # list of float32 [kz,ky,kx], odd sizes
    psftype: int
    iterations: int
    lam: float
    block: tuple | None  # (bx, by, bz) or None for one block
    ground_truth: np.ndarray | None = None

    @property
    def shape(self):
        return self.views[0].shape

    @property
    def dims_xyz(self):
        z, y, x = self.views[0].shape
        return (x, y, z)

    @property
    def n_voxels(self):
        return int(np.prod(self.views[0].shape))


def rotation_y(angle_deg: float) -> np.ndarray:
    """Rotation about y acting on (x, y, z) column vectors."""
    t = math.radians(angle_deg)
    c, s = math.cos(t), math.sin(t)
    return np.array([[c, 0.0, s], [0.0, 1.0, 0.0], [-s, 0.0, c]])


def transformed_psf_size(size_xyz, rot: np.ndarray):
    """Bounding-box size of a rotated PSF, forced odd (ExtractPSF.transformPSF, :325-364)."""
    ext = np.abs(rot) @ (np.asarray(size_xyz, dtype=np.float64) - 1.0)
    out = []
    for e in ext:
        n = int(e + 1e-9) + 1
        if n % 2 == 0:
            n += 1
        out.append(n)
    return tuple(out)


def gaussian_psf(sigma_xyz, size_xyz, angle_deg: float = 0.0) -> np.ndarray:
    """Anisotropic Gaussian rotated about y, evaluated on an odd grid centred at size//2.

    The size is the transformed size of ``size_xyz`` under the rotation; the result has unit
    sum (FP64) and is returned as float32 ``[z, y, x]``.
    """
    rot = rotation_y(angle_deg)
    nx, ny, nz = transformed_psf_size(size_xyz, rot)
    z, y, x = np.meshgrid(
        np.arange(nz) - nz // 2, np.arange(ny) - ny // 2, np.arange(nx) - nx // 2, indexing="ij"
    )
    d = np.stack([x, y, z], axis=-1).astype(np.float64)  # (..., 3) in the fused frame
    local = d @ rot  # rot^T d for row vectors
    s = np.asarray(sigma_xyz, dtype=np.float64)
    g = np.exp(-0.5 * np.sum((local / s) ** 2, axis=-1))
    g /= g.sum()
    return g.astype(np.float32)


def blobs(shape_zyx, n_blobs, sigma_range, peak_range, background, rng) -> np.ndarray:
    """Ground truth: isotropic Gaussian blobs added onto a constant background (float64)."""
    vol = np.full(shape_zyx, float(background), dtype=np.float64)
    nz, ny, nx = shape_zyx
    for _ in range(n_blobs):
        cz, cy, cx = rng.uniform(0, nz), rng.uniform(0, ny), rng.uniform(0, nx)
        sig = rng.uniform(*sigma_range)
        peak = rng.uniform(*peak_range)
        r = int(math.ceil(4 * sig))
        z0, z1 = max(0, int(cz) - r), min(nz, int(cz) + r + 1)
        y0, y1 = max(0, int(cy) - r), min(ny, int(cy) + r + 1)
        x0, x1 = max(0, int(cx) - r), min(nx, int(cx) + r + 1)
        if z0 >= z1 or y0 >= y1 or x0 >= x1:
            continue
        zz, yy, xx = np.meshgrid(
            np.arange(z0, z1), np.arange(y0, y1), np.arange(x0, x1), indexing="ij"
        )
        d2 = (zz - cz) ** 2 + (yy - cy) ** 2 + (xx - cx) ** 2
        vol[z0:z1, y0:y1, x0:x1] += peak * np.exp(-0.5 * d2 / sig**2)
    return vol


def _mirror_single_index(idx: np.ndarray, n: int) -> np.ndarray:
    """Index map of imglib2's mirror-single out-of-bounds strategy (-1 -> 1, n -> n-2)."""
    if n == 1:
        return np.zeros_like(idx)
    period = 2 * n - 2
    m = np.mod(idx, period)
    return np.where(m < n, m, period - m)


def blur_mirror(vol: np.ndarray, psf: np.ndarray) -> np.ndarray:
    """Linear convolution of the mirror-single extended volume with a centred kernel (FP64)."""
    kz, ky, kx = psf.shape
    hz, hy, hx = kz // 2, ky // 2, kx // 2
    nz, ny, nx = vol.shape
    ext = vol[
        np.ix_(
            _mirror_single_index(np.arange(-hz, nz + hz), nz),
            _mirror_single_index(np.arange(-hy, ny + hy), ny),
            _mirror_single_index(np.arange(-hx, nx + hx), nx),
        )
    ].astype(np.float64)
    shape = [ext.shape[i] + psf.shape[i] - 1 for i in range(3)]
    f = np.fft.rfftn(ext, shape, axes=(0, 1, 2)) * np.fft.rfftn(psf.astype(np.float64), shape, axes=(0, 1, 2))
    full = np.fft.irfftn(f, shape, axes=(0, 1, 2))
    return full[kz - 1 : kz - 1 + nz, ky - 1 : ky - 1 + ny, kx - 1 : kx - 1 + nx]


_BLEND_LUT = np.array(
    [(math.cos((1 - i / 1000.0) * math.pi) + 1) / 2 for i in range(1001)], dtype=np.float64
)


def blending_weight(q_xyz: np.ndarray, dims_xyz, border_xyz, range_xyz) -> np.ndarray:
    """Cosine blending weight at real positions (BlendingRealRandomAccess.computeWeight :91-121),
    for generating test volumes only: the table holds exact k/1000 values and the index rounds
    half to even, where the reference accumulates d and rounds half up (the GPU input
    preparation follows the reference bit for bit)."""
    w = np.ones(q_xyz.shape[:-1], dtype=np.float32)
    zero = np.zeros(q_xyz.shape[:-1], dtype=bool)
    for d in range(3):
        l = q_xyz[..., d].astype(np.float32)
        dm1 = np.float32(dims_xyz[d] - 1)
        dist = np.maximum(0, np.minimum(l - border_xyz[d], dm1 - l - border_xyz[d])).astype(np.float32)
        zero |= dist == 0
        rel = dist / np.float32(range_xyz[d])
        lut = _BLEND_LUT[np.clip(np.round(rel.astype(np.float64) * 1000.0), 0, 1000).astype(np.int64)]
        w = np.where(rel < 1, (w * lut).astype(np.float32), w)
    return np.where(zero, np.float32(0), w).astype(np.float32)


def view_weight(dims_xyz, angle_deg, border=(-8, -8, -3), blend=(12, 12, 12)) -> np.ndarray:
    """Blending weight of a view whose stack is the fused box rotated about its centre."""
    nx, ny, nz = dims_xyz
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    c = np.array([(nx - 1) / 2.0, (ny - 1) / 2.0, (nz - 1) / 2.0])
    p = np.stack([x, y, z], axis=-1).astype(np.float64) - c
    q = p @ rotation_y(angle_deg) + c  # rot^T (p - c) + c
    return blending_weight(q, dims_xyz, border, blend)


def normalise_weights_virtual(weights, osem=1.0):
    """VIRTUAL weight normalisation: w / (sum > 1 ? sum : 1), then min(1, w * osem)."""
    s = np.zeros_like(weights[0], dtype=np.float64)
    for w in weights:
        s += w
    norm = np.where(s > 1, s, 1.0).astype(np.float32)
    out = []
    for w in weights:
        v = w.astype(np.float64) / norm.astype(np.float64)
        out.append(np.minimum(1.0, v * osem).astype(np.float32))
    return out


def simulate_views(gt: np.ndarray, psfs, rng, coverage=None):
    """img_v = max(minValue, Poisson(gt * P_v)) inside the view, 0 outside."""
    views = []
    for i, p in enumerate(psfs):
        blurred = np.maximum(blur_mirror(gt, p), 0.0)
        img = rng.poisson(blurred).astype(np.float32)
        img = np.maximum(img, MIN_VALUE)
        if coverage is not None:
            img = np.where(coverage[i], img, np.float32(0)).astype(np.float32)
        views.append(img.astype(np.float32))
    return views


def _rng(cfg_id: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(1000 + cfg_id))


def make_problem(
    cfg_id: int,
    shape_xyz=None,
    psf_size_xyz=None,
    n_blobs=None,
    iterations=None,
    psftype=None,
    lam=None,
    block=None,
    n_views=None,
) -> Problem:
    """Build one of the five seeded configurations, optionally shrunk for fast tests.

    1: 2 views (0, 90 deg), 128x128x64, PSF 9x9x25 sigma (1.2,1.2,4), weights 1, INDEPENDENT,
       10 iterations, one block.
    2: 4 views (0/45/90/135 deg), 256x256x192, PSF 15x15x41 sigma (1.5,1.5,5), cosine
       blending + VIRTUAL weights, EFFICIENT_BAYESIAN, 128^3 blocks, 20 iterations.
    3: 6 views each cropped to a random box with sides U[96,256] inside a 256^3 box
       (img = 0 and w = 0 outside the crop), PSF as cfg 2, 20 iterations.
    4: 4 views, 512x512x256, PSF 31x31x61 sigma (2,2,7), 10 iterations.
    5: 4 views, 192^3, 500 beads (sigma 0.7, peak U[500,2000]), PSF 31x31x61.
    """
    rng = _rng(cfg_id)
    cfg = {
        1: dict(shape=(128, 128, 64), psf=(9, 9, 25), sigma=(1.2, 1.2, 4.0), angles=[0, 90],
                blobs=200, bsig=(1.5, 3.0), peak=(100, 1000), bg=10.0, it=10,
                ptype=INDEPENDENT, weights="ones", block=None),
        2: dict(shape=(256, 256, 192), psf=(15, 15, 41), sigma=(1.5, 1.5, 5.0),
                angles=[0, 45, 90, 135], blobs=200, bsig=(1.5, 3.0), peak=(100, 1000), bg=10.0,
                it=20, ptype=EFFICIENT_BAYESIAN, weights="blend", block=(128, 128, 128)),
        3: dict(shape=(256, 256, 256), psf=(15, 15, 41), sigma=(1.5, 1.5, 5.0),
                angles=[0, 30, 60, 90, 120, 150], blobs=200, bsig=(1.5, 3.0), peak=(100, 1000),
                bg=10.0, it=20, ptype=EFFICIENT_BAYESIAN, weights="crop", block=(128, 128, 128)),
        4: dict(shape=(512, 512, 256), psf=(31, 31, 61), sigma=(2.0, 2.0, 7.0),
                angles=[0, 45, 90, 135], blobs=1600, bsig=(1.5, 3.0), peak=(100, 1000), bg=10.0,
                it=10, ptype=EFFICIENT_BAYESIAN, weights="blend", block=None),
        5: dict(shape=(192, 192, 192), psf=(31, 31, 61), sigma=(2.0, 2.0, 7.0),
                angles=[0, 45, 90, 135], blobs=500, bsig=(0.7, 0.7), peak=(500, 2000), bg=10.0,
                it=10, ptype=EFFICIENT_BAYESIAN, weights="blend", block=None),
    }[cfg_id]
    if shape_xyz is not None:
        cfg["shape"] = tuple(shape_xyz)
    if psf_size_xyz is not None:
        cfg["psf"] = tuple(psf_size_xyz)
    if n_blobs is not None:
        cfg["blobs"] = n_blobs
    if n_views is not None:
        cfg["angles"] = cfg["angles"][:n_views]
    nx, ny, nz = cfg["shape"]
    shape_zyx = (nz, ny, nx)
    gt = blobs(shape_zyx, cfg["blobs"], cfg["bsig"], cfg["peak"], cfg["bg"], rng)
    psfs = [gaussian_psf(cfg["sigma"], cfg["psf"], a) for a in cfg["angles"]]
    coverage = None
    if cfg["weights"] == "crop":
        coverage = []
        for _ in cfg["angles"]:
            m = np.zeros(shape_zyx, dtype=bool)
            # sides U[96, 256] on a 256 box; the same fractions on a shrunk box
            side = [int(rng.integers(max(4, (96 * s) // 256), max(5, (256 * s) // 256) + 1)) for s in (nx, ny, nz)]
            side = [min(sd, s) for sd, s in zip(side, (nx, ny, nz))]
            off = [int(rng.integers(0, s - sd + 1)) for s, sd in zip((nx, ny, nz), side)]
            m[off[2]:off[2] + side[2], off[1]:off[1] + side[1], off[0]:off[0] + side[0]] = True
            coverage.append(m)
    views = simulate_views(gt, psfs, rng, coverage)
    if cfg["weights"] == "ones":
        weights = [np.ones(shape_zyx, dtype=np.float32) for _ in psfs]
    else:
        raw = [view_weight(cfg["shape"], a) for a in cfg["angles"]]
        if coverage is not None:
            raw = [np.where(c, w, np.float32(0)).astype(np.float32) for w, c in zip(raw, coverage)]
        weights = normalise_weights_virtual(raw)
    return Problem(
        name=f"cfg{cfg_id}",
        views=views,
        weights=weights,
        psfs=psfs,
        psftype=cfg["ptype"] if psftype is None else psftype,
        iterations=cfg["it"] if iterations is None else iterations,
        lam=0.006 if lam is None else lam,
        block=cfg["block"] if block is None else (None if block == "none" else block),
        ground_truth=gt.astype(np.float32),
    )
