"""PSF pipeline on the GPU against the oracle: extraction from bead neighbourhoods (periodic
trilinear, summed over the locations), normalisation, the transform into the fused frame and
ExtractPSF's per-view bookkeeping.  FP32 interpolation: max abs error <= 1e-5 of the output's
max."""
import math

import numpy as np
import pytest

from oracle import mvdecon_oracle as O
from spim_registration_gb300 import ExtractPSF
from spim_registration_gb300.psf import extract_psf_local, transform_psf

pytestmark = pytest.mark.gpu


def _rot_y(deg, scale=(1.0, 1.0, 1.0), shift=(0.0, 0.0, 0.0)):
    t = math.radians(deg)
    r = np.array([[math.cos(t), 0, math.sin(t)], [0, 1, 0], [-math.sin(t), 0, math.cos(t)]]) @ np.diag(scale)
    return np.concatenate([r, np.asarray(shift, dtype=np.float64)[:, None]], axis=1).ravel()


def _close(got, want, tol=1e-5):
    err = np.abs(got.astype(np.float64) - want).max() / max(np.abs(want).max(), 1e-30)
    assert err <= tol, err


def _beads(rng, shape_zyx, n):
    img = (rng.random(shape_zyx) * 5).astype(np.float32)
    locs = []
    for _ in range(n):
        c = [rng.uniform(0, s) for s in shape_zyx[::-1]]  # anywhere: boxes wrap at the border
        locs.append(c)
        z, y, x = np.meshgrid(*[np.arange(s) for s in shape_zyx], indexing="ij")
        img += (300 * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2) / 2.0 - (z - c[2]) ** 2 / 8.0)).astype(np.float32)
    return img, locs


@pytest.mark.parametrize("normalize", [False, True])
def test_extraction_matches_oracle(normalize):
    rng = np.random.default_rng(11)
    img, locs = _beads(rng, (40, 48, 56), 25)
    got = extract_psf_local(img, locs, (9, 11, 13), normalize=normalize)
    want = O.extract_psf_local(img, locs, (9, 11, 13), normalize=normalize)
    assert got.shape == (13, 11, 9)
    _close(got, want)


@pytest.mark.parametrize("deg,scale", [(0, (1, 1, 1)), (30, (1, 1, 2.5)), (90, (1, 1, 1.7)), (137, (1.2, 0.9, 2))])
def test_transform_matches_oracle(deg, scale):
    rng = np.random.default_rng(deg)
    psf = rng.random((21, 11, 9)).astype(np.float32)
    m = _rot_y(deg, scale, (3.0, -2.0, 7.5))
    got = transform_psf(psf, m)
    dims, off = O.transformed_psf_size((9, 11, 21), m)
    want = O.transform_psf(psf, m, dims, off)
    assert got.shape == tuple(dims[::-1])
    _close(got, want)


def test_extract_psf_class_per_view_and_average():
    rng = np.random.default_rng(12)
    img, locs = _beads(rng, (32, 36, 40), 12)
    ex = ExtractPSF()
    models = {"a": _rot_y(0), "b": _rot_y(45, (1, 1, 2)), "c": _rot_y(90, (1, 1, 1.5))}
    for v, m in models.items():
        ex.extractNextImg(img, v, m, locs, (7, 7, 11))
    assert ex.getViewIdsForPSFs() == list(models)
    want_orig = O.extract_psf_local(img, locs, (7, 7, 11), normalize=True)
    for v, m in models.items():
        _close(ex.getInputCalibrationPSFs()[v], want_orig)
        dims, off = O.transformed_psf_size((7, 7, 11), m)
        _close(ex.getTransformedPSF(v), O.transform_psf(want_orig, m, dims, off))
    avg = ex.computeAverageTransformedPSF()
    assert avg.shape == tuple(ex.computeMaxDimTransformedPSF()[::-1])
    assert avg.sum() == pytest.approx(sum(p.sum() for p in ex.getPSFMap().values()), rel=1e-5)
