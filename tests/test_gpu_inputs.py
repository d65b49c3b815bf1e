"""Input preparation on the GPU against the oracle: a view resampled into the fused box
(TransformInput), its blending weight (TransformWeights + BlendingRealRandomAccess) and the
VIRTUAL weight normalisation with the OSEM factor (WeightNormalizer).

The GPU evaluates the inverse transform in float, the oracle in double, so voxels whose view
position lies within 1e-3 of the view's border (the inside test) are left out of the value
comparison; the blending lookup table is piecewise constant in steps of 0.001, so weights are
compared to 3e-3 absolute (most are identical).
"""
import math

import numpy as np
import pytest

from oracle import mvdecon_oracle as O
from spim_registration_gb300 import native

pytestmark = pytest.mark.gpu


def _affine(angle_deg, scale_xyz, shift_xyz):
    t = math.radians(angle_deg)
    c, s = math.cos(t), math.sin(t)
    rot = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
    m = rot @ np.diag(scale_xyz)
    return np.concatenate([m, np.asarray(shift_xyz, dtype=np.float64)[:, None]], axis=1).ravel()


@pytest.mark.parametrize("angle,scale", [(0.0, (1, 1, 1)), (30.0, (1, 1, 2.0)), (90.0, (1.0, 1.0, 1.5))])
def test_transform_view_matches_oracle(angle, scale):
    torch = pytest.importorskip("torch")
    lib = native.load()
    rng = np.random.default_rng(3)
    view = (rng.random((18, 22, 26)) * 100 + 1).astype(np.float32)  # z, y, x
    affine = _affine(angle, scale, (14.25, 3.375, 9.125))  # fractional: no position exactly on the border
    out_shape = (40, 30, 44)  # z, y, x
    offset = (-6, -2, -5)
    border, blend = (-8.0, -8.0, -3.0), (12.0, 12.0, 12.0)
    dv = torch.from_numpy(view).cuda()
    oimg = torch.full(out_shape, float("nan"), device="cuda")
    oblend = torch.full(out_shape, float("nan"), device="cuda")
    st = lib.mvd_transform_view(dv.data_ptr(), native.iarr([26, 22, 18]), (native.ctypes.c_double * 12)(*affine),
                                native.iarr(offset), native.iarr([44, 30, 40]), oimg.data_ptr(), oblend.data_ptr(),
                                (native.ctypes.c_float * 3)(*border), (native.ctypes.c_float * 3)(*blend), 0, None)
    native.check(st)
    torch.cuda.synchronize()
    got = oimg.cpu().numpy().astype(np.float64)
    want = O.transform_input(view, affine, offset, out_shape)
    t = O._view_positions(affine, offset, out_shape)
    size = np.array([26, 22, 18])
    margin = np.minimum(np.abs(t), np.abs(t - size)).min(axis=-1)
    safe = margin > 1e-3
    assert safe.mean() > 0.9
    inside = want > 0
    assert inside[safe].any() and (~inside[safe]).any() or angle == 0.0
    assert np.array_equal(got[safe] > 0, inside[safe])
    rel = np.abs(got - want)[safe].max() / np.abs(want).max()
    assert rel < 1e-5, rel
    wb = O.transform_weights(view.shape, affine, offset, out_shape, border, blend)
    gb = oblend.cpu().numpy()
    assert np.isfinite(gb).all()
    assert np.abs(gb - wb).max() < 3e-3
    assert np.mean(gb == wb) > 0.98


def _blend_on_device(lib, torch, view_zyx, out_zyx, border, blend, offset=(0, 0, 0)):
    eye = [1.0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0, 0]
    dv = torch.ones(view_zyx, dtype=torch.float32, device="cuda")
    oblend = torch.full(out_zyx, float("nan"), device="cuda")
    vz, vy, vx = view_zyx
    oz, oy, ox = out_zyx
    native.check(lib.mvd_transform_view(dv.data_ptr(), native.iarr([vx, vy, vz]), (native.ctypes.c_double * 12)(*eye),
                                        native.iarr(list(offset)), native.iarr([ox, oy, oz]), None,
                                        oblend.data_ptr(), (native.ctypes.c_float * 3)(*border),
                                        (native.ctypes.c_float * 3)(*blend), 0, None))
    torch.cuda.synchronize()
    return oblend.cpu().numpy()


@pytest.mark.parametrize("turn", ["x", "z"])
def test_exact_quarter_turn_is_a_transpose(turn):
    """A registration turning the view by exactly 90 degrees about y maps voxel centres onto
    voxel centres, and the float inverse is exact: image and weight are the view's own values,
    transposed and flipped, bit for bit.  The turn makes view x run along output z, which the
    z-fast resampling kernel takes; "x" is the unturned view through the x-fast kernel."""
    torch = pytest.importorskip("torch")
    lib = native.load()
    rng = np.random.default_rng(9)
    sz, sy, sx = 37, 21, 45  # odd sizes: partial tiles in both kernels
    view = (rng.random((sz, sy, sx)) * 100 + 1).astype(np.float32)
    if turn == "z":
        affine, out_shape = [0, 0, 1, 0, 0, 1, 0, 0, -1, 0, 0, sx - 1], (sx, sy, sz)
        want = np.transpose(view, (2, 1, 0))[::-1]
    else:
        affine, out_shape = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], (sz, sy, sx)
        want = view
    border, blend = (0.5, -2.0, 1.0), (9.0, 6.5, 7.25)
    eye = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    w_view = O.transform_weights(view.shape, eye, (0, 0, 0), view.shape, border, blend)
    want_w = np.transpose(w_view, (2, 1, 0))[::-1] if turn == "z" else w_view
    dv = torch.from_numpy(view).cuda()
    oimg = torch.full(out_shape, float("nan"), device="cuda")
    oblend = torch.full(out_shape, float("nan"), device="cuda")
    oz, oy, ox = out_shape
    native.check(lib.mvd_transform_view(dv.data_ptr(), native.iarr([sx, sy, sz]),
                                        (native.ctypes.c_double * 12)(*[float(a) for a in affine]),
                                        native.iarr([0, 0, 0]), native.iarr([ox, oy, oz]), oimg.data_ptr(),
                                        oblend.data_ptr(), (native.ctypes.c_float * 3)(*border),
                                        (native.ctypes.c_float * 3)(*blend), 0, None))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(oimg.cpu().numpy(), want)
    np.testing.assert_array_equal(oblend.cpu().numpy(), want_w)


def test_blending_weight_arithmetic_is_bit_exact():
    """With the identity registration the kernel and the oracle see the same float positions,
    so the weights must agree bit for bit: the lookup index (Math.round of the double product
    rel * 1000) and minDistance *= lookUp[i] (float times double, rounded twice) over products
    of two and three table entries, with fractional borders and blending ranges."""
    torch = pytest.importorskip("torch")
    lib = native.load()
    view, border, blend = (61, 70, 83), (0.3, -1.7, 2.1), (40.3, 35.7, 30.1)
    got = _blend_on_device(lib, torch, view, view, border, blend)
    want = O.transform_weights(view, [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], (0, 0, 0), view, border, blend)
    assert (want > 0).mean() > 0.8 and len(np.unique(want)) > 10000
    np.testing.assert_array_equal(got, want)


def test_blending_lookup_index_at_half_steps():
    """rel = (x - 0.5) / 1000: every rel * 1000 lies within a float rounding of k + 0.5, the
    boundary between two table entries."""
    torch = pytest.importorskip("torch")
    lib = native.load()
    view, border, blend = (3, 3, 2003), (0.5, -5.0, -5.0), (1000.0, 1.0, 1.0)
    got = _blend_on_device(lib, torch, view, view, border, blend)
    want = O.transform_weights(view, [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], (0, 0, 0), view, border, blend)
    np.testing.assert_array_equal(got, want)
    row = want[1, 1]
    assert row[0] == 0 and np.all(np.diff(row[:1001]) >= 0)


def _weights(rng, shape, zero_frac):
    # a mix of generic floats and products of blending-table values, with zeros; 3% tiny
    # values (2^-40 .. 2^-70) and 1% denormals spread the views' exponents beyond what the
    # kernel's integer sum covers, so those voxels take its double sum
    lut = O._BLEND_LUT.astype(np.float32)
    a = rng.random(shape).astype(np.float32) ** 2
    b = lut[rng.integers(0, 1001, shape)] * lut[rng.integers(0, 1001, shape)]
    tiny = np.ldexp(rng.random(shape), -rng.integers(40, 71, shape)).astype(np.float32)
    den = (rng.integers(1, 1 << 23, shape).astype(np.uint32)).view(np.float32)
    u = rng.random(shape)
    w = np.where(u < 0.5, a, b)
    w = np.where(u > 0.97, tiny, np.where(u > 0.96, den, w))
    return np.where(rng.random(shape) < zero_frac, 0, w).astype(np.float32)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("osem", [1.0, 1.7, 157 / 66, 2.0])
def test_normalize_weights_equal_the_reference_arithmetic(mode, osem):
    """Bit-equal to the reference's double arithmetic, NaN positions included (PRECOMPUTED
    divides 0 by 0 where no view has weight).  osem 1.7 makes ~5% of the products exact
    rational ties, which the certified float pairs hand to the double pass."""
    torch = pytest.importorskip("torch")
    lib = native.load()
    rng = np.random.default_rng(4)
    ws = [_weights(rng, (40, 48, 52), 0.3) for _ in range(4)]
    want = (O.normalize_weights_virtual if mode == 0 else O.normalize_weights_precomputed)(ws, osem)
    dws = [torch.from_numpy(w).cuda() for w in ws]
    ptrs = (native.ctypes.c_void_p * 4)(*[d.data_ptr() for d in dws])
    native.check(lib.mvd_normalize_weights(ptrs, 4, ws[0].size, osem, mode, 0, None))
    torch.cuda.synchronize()
    for d, w in zip(dws, want):
        np.testing.assert_array_equal(d.cpu().numpy(), w)


@pytest.mark.parametrize("portions", [1, 7, 32])
def test_weight_overlap_matches_oracle(portions):
    torch = pytest.importorskip("torch")
    from spim_registration_gb300 import WeightNormalizer

    rng = np.random.default_rng(7)
    shape = (37, 29, 23)  # odd sizes: portion borders fall inside warps
    ws = [np.where(rng.random(shape) < 0.3, 0, rng.random(shape)).astype(np.float32) for _ in range(4)]
    mn, avg = O.weight_overlap(ws, portions)
    wn = WeightNormalizer([torch.from_numpy(w).cuda() for w in ws], num_portions=portions)
    assert wn.process()
    assert wn.getMinOverlappingViews() == mn
    assert wn.getAvgOverlappingViews() == pytest.approx(avg, rel=1e-12)
    ws[1][:] = 0.5  # every voxel covered at least once
    wn = WeightNormalizer([torch.from_numpy(w).cuda() for w in ws], num_portions=portions)
    wn.process()
    assert wn.getMinOverlappingViews() == O.weight_overlap(ws, portions)[0] >= 1


def test_raw_views_to_deconvolution_on_the_device():
    """Raw views + registrations -> resampled views and blending weights -> overlap statistics
    -> VIRTUAL normalisation with the average-overlap OSEM factor -> deconvolution from the
    device tensors; the oracle runs the same chain in FP64."""
    torch = pytest.importorskip("torch")
    from spim_registration_gb300 import PSFTYPE, Deconvolution, WeightNormalizer, transform_input
    from spim_registration_gb300 import synthetic as S
    from tests.helpers import rel_l2

    rng = np.random.default_rng(8)
    box = (36, 40, 44)  # z, y, x
    offset = (-3, -2, -4)
    raw, affines = [], []
    for angle in (0.0, 40.0, 90.0):
        raw.append((S.gaussian_psf((3.0, 3.0, 3.0), (41, 37, 33), 0.0) * 5000 + rng.random((33, 37, 41)) * 10
                    + 1).astype(np.float32))
        c, s_ = math.cos(math.radians(angle)), math.sin(math.radians(angle))
        # the view centre (20, 18, 16 * 1.25) lands near the box centre (18, 18, 15), off the grid
        shift = (18.25 - (20 * c + 20 * s_), 0.375, 15.125 - (-20 * s_ + 20 * c))
        affines.append(_affine(angle, (1.0, 1.0, 1.25), shift))
    border, blend = (0.0, 0.0, 0.0), (8.0, 8.0, 6.0)
    psfs = [(lambda k: (k / k.sum()).astype(np.float32))(S.gaussian_psf((1.2, 1.2, 2.5), (7, 7, 11), 0.0))
            for _ in raw]
    dev_views, dev_weights = [], []
    for r, a in zip(raw, affines):
        img, w = transform_input(r, a, offset, box, border, blend)
        dev_views.append(img)
        dev_weights.append(w)
    wn = WeightNormalizer(dev_weights, num_portions=8)
    wn.process()
    osem = wn.osem_speedup(2)
    wn.apply(osem)
    d = Deconvolution(dev_views, dev_weights, psfs, PSFTYPE.EFFICIENT_BAYESIAN, 0.006)
    d.run(3)
    got = d.get_psi()

    views = [O.transform_input(r, a, offset, box).astype(np.float32) for r, a in zip(raw, affines)]
    weights = [O.transform_weights(r.shape, a, offset, box, border, blend) for r, a in zip(raw, affines)]
    mn, avg = O.weight_overlap(weights, 8)
    assert wn.getMinOverlappingViews() == mn and osem == pytest.approx(max(1.0, avg), rel=1e-12)
    weights = O.normalize_weights_virtual(weights, max(1.0, avg))
    for dv, v in zip(dev_views, views):
        assert rel_l2(dv.cpu().numpy(), v) < 1e-5
    p = S.Problem("raw", views, weights, psfs, int(PSFTYPE.EFFICIENT_BAYESIAN), 3, 0.006, None)
    ref, _ = O.deconvolve(p, arith="f64", block=None, mask=False)
    assert rel_l2(got, ref) < 1e-4, rel_l2(got, ref)


def test_transform_view_rejects_singular_affines():
    lib = native.load()
    st = lib.mvd_transform_view(1, native.iarr([4, 4, 4]), (native.ctypes.c_double * 12)(*([0.0] * 12)),
                                native.iarr([0, 0, 0]), native.iarr([4, 4, 4]), 1, None, None, None, 0, None)
    assert st == 1 and "singular" in lib.mvd_last_error().decode()
