"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests or golden vectors for this path, so the oracle is pinned by
mathematical identities of the restated algorithm and by the committed golden fixtures that
tests/golden/make_golden.py generates from it.
"""
import math

import numpy as np
import pytest

from oracle import mvdecon_oracle as O
from spim_registration_gb300 import synthetic as S


def rng(seed=0):
    return np.random.default_rng(seed)


@pytest.mark.parametrize("mode,value", [(O.MIRROR, 0.0), (O.VALUE, 1.0), (O.VALUE, 0.0)])
@pytest.mark.parametrize("shape,kshape", [((16, 16, 16), (5, 5, 9)), ((11, 7, 13), (3, 5, 7)), ((5, 6, 4), (7, 3, 9))])
def test_fft_conv_equals_direct_conv(mode, value, shape, kshape):
    r = rng(1)
    img = r.random(shape)
    k = r.random(kshape)
    a = O.conv_extended(img, k, mode, value)
    b = O.conv_direct(img, k, mode, value)
    assert np.abs(a - b).max() < 1e-10 * max(1.0, np.abs(b).max())


def test_delta_psf_is_identity():
    img = rng(2).random((9, 10, 11))
    k = np.zeros((5, 3, 7))
    k[2, 1, 3] = 1.0
    for mode in (O.MIRROR, O.VALUE):
        np.testing.assert_allclose(O.conv_extended(img, k, mode, 1.0), img, atol=1e-12)


def test_delta_image_gives_centred_psf():
    img = np.zeros((21, 21, 21))
    img[10, 10, 10] = 1.0
    k = rng(3).random((5, 7, 9))
    out = O.conv_extended(img, k, O.VALUE, 0.0)
    np.testing.assert_allclose(out[8:13, 7:14, 6:15], k, atol=1e-12)
    assert abs(out.sum() - k.sum()) < 1e-10


def test_mirror_single_index_map():
    n = 5
    idx = np.arange(-6, 12)
    m = O.mirror_single_index(idx, n)
    # -1 -> 1, n -> n-2, period 2n-2
    assert m[idx == -1][0] == 1 and m[idx == n][0] == n - 2
    assert np.all((m >= 0) & (m < n))
    assert np.array_equal(O.mirror_single_index(idx + 2 * n - 2, n), m)


def test_mirror_kernel_odd_is_flip_even_keeps_middle():
    a = np.arange(3 * 5 * 7, dtype=np.float64).reshape(3, 5, 7)
    np.testing.assert_array_equal(O.mirror(a), a[::-1, ::-1, ::-1])
    b = np.arange(4, dtype=np.float64).reshape(1, 1, 4)
    # Mirror.java swaps p<->n-1-p for p <= n/2: the middle pair of an even axis is swapped twice
    np.testing.assert_array_equal(O.mirror(b)[0, 0], [3, 1, 2, 0])


def test_blocked_equals_single_block():
    r = rng(4)
    img = r.random((20, 23, 26))
    k = r.random((7, 5, 9))
    whole = O.conv_extended(img, k, O.MIRROR)
    for block in [(12, 10, 14), (26, 23, 20), (9, 5, 7)]:
        blk = O.convolve_blocked(img, k, block, O.MIRROR)
        np.testing.assert_allclose(blk, whole, rtol=1e-12, atol=1e-12)
    whole1 = O.conv_extended(img, k, O.VALUE, 1.0)
    np.testing.assert_allclose(O.convolve_blocked(img, k, (12, 10, 14), O.VALUE, 1.0), whole1, rtol=1e-12, atol=1e-12)


def test_block_generator_matches_reference_rules():
    blocks = O.divide_into_blocks((100, 50, 30), (9, 9, 15), (32, 32, 32))
    eff = (24, 24, 18)
    assert len(blocks) == 5 * 3 * 2
    covered = np.zeros((30, 50, 100), dtype=int)
    for b in blocks:
        for d in range(3):
            assert b["offset"][d] == b["eff_offset"][d] - (9, 9, 15)[d] // 2
            assert b["eff_size"][d] <= eff[d]
        ex, ey, ez = b["eff_offset"]
        sx, sy, sz = b["eff_size"]
        covered[ez:ez + sz, ey:ey + sy, ex:ex + sx] += 1
    assert np.all(covered == 1)
    with pytest.raises(ValueError):
        O.divide_into_blocks((10, 10, 10), (9, 9, 15), (8, 32, 32))


def test_rl_fixed_point():
    """img = psi (*) P, w = 1, lambda = 0: a view stage leaves psi unchanged."""
    r = rng(5)
    psi = 10 + 50 * r.random((12, 14, 16))
    k = S.gaussian_psf((1.2, 1.0, 2.0), (5, 5, 9))
    img = O.conv_extended(psi, k, O.MIRROR)
    d = O.Deconvolution([img.astype(np.float32)], [np.ones_like(img, dtype=np.float32)], [k], O.INDEPENDENT, 0.0,
                        psi0=psi)
    # kernel2 = mirror(kernel1): the quotient is 1 everywhere, conv2 of 1 is 1 (value-1 border)
    d.run_view(0)
    np.testing.assert_allclose(d.psi, psi, rtol=1e-6)


def test_normalisation_quirk_counts_portion_zero_twice():
    k = np.ones((3, 3, 3), dtype=np.float32)
    s = O.sum_img(k)
    sq = O.sum_img(k, quirk_threads=2)  # 4 portions of 27 voxels: portion 0 has 6
    assert s == 27 and sq == 33
    assert abs(O.norm_img(k).sum() - 1) < 1e-12


def test_compound_kernels_are_unit_sum_and_shaped():
    psfs = [S.gaussian_psf((1.2, 1.2, 3.0), (7, 7, 11), a) for a in (0, 60, 120)]
    for ptype in (O.EFFICIENT_BAYESIAN, O.OPTIMIZATION_I, O.OPTIMIZATION_II, O.INDEPENDENT):
        k1, k2 = O.prepare_kernels(psfs, ptype)
        for a, b, p in zip(k1, k2, psfs):
            assert a.shape == p.shape and b.shape == p.shape
            assert abs(b.sum() - 1) < 1e-9 and abs(a.sum() - 1) < 1e-9
    # one view: every type reduces to the mirrored kernel (MVDeconFFT.java:197-201)
    k1, k2 = O.prepare_kernels(psfs[:1], O.EFFICIENT_BAYESIAN)
    np.testing.assert_allclose(k2[0], O.mirror(k1[0]))


def test_first_iteration_average_and_mask():
    a = np.array([[[0, 2, 4]]], dtype=np.float32)
    b = np.array([[[0, 0, 6]]], dtype=np.float32)
    avg, count = O.first_iteration([a, b])
    assert avg == pytest.approx((2 + 5) / 2)
    np.testing.assert_array_equal(count[0, 0], [0, 1, 2])


def test_update_rules_match_java_float_semantics():
    psi = np.array([1.0, 2.0, 0.5, 3.0], dtype=np.float32)
    integral = np.array([2.0, 0.0, np.nan, 1.0], dtype=np.float32)
    w = np.array([1.0, 1.0, 1.0, 0.5], dtype=np.float32)
    new, s, m = O.compute_final_values(psi, integral, w, 0.006, "f32")
    tik = lambda v: (np.sqrt(1 + 2 * 0.006 * v) - 1) / 0.006  # noqa: E731
    assert new[0] == np.float32(tik(2.0))
    f = np.float32
    mv = f(1e-4)
    # value 0 -> minValue, NaN -> minValue; then last + (next - last) * w in float
    assert new[1] == f(f(2.0) + f(f(mv - f(2.0)) * f(1.0)))
    assert new[2] == f(f(0.5) + f(f(mv - f(0.5)) * f(1.0)))
    assert new[3] == np.float32(3.0 + (np.float32(tik(3.0)) - 3.0) * 0.5)
    assert s == pytest.approx(float(np.abs(new - psi).astype(np.float64).sum()))


def test_deconvolution_f32_tracks_f64():
    p = S.make_problem(1, shape_xyz=(40, 36, 24), psf_size_xyz=(7, 7, 11), n_blobs=15, iterations=3)
    a, _ = O.deconvolve(p, arith="f64")
    b, _ = O.deconvolve(p, arith="f32")
    assert np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-5


def test_blocked_deconvolution_equals_whole():
    p = S.make_problem(2, shape_xyz=(40, 36, 28), psf_size_xyz=(5, 5, 9), n_blobs=15, iterations=2)
    a, _ = O.deconvolve(p, block=None)
    b, _ = O.deconvolve(p, block=(24, 20, 20))
    np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-10)


def test_nll_gradient_matches_central_differences():
    p = S.make_problem(5, shape_xyz=(14, 12, 10), psf_size_xyz=(3, 3, 5), n_blobs=6, n_views=2)
    psi = p.views[0].astype(np.float64) * 0.9 + 3
    psfs = [q.astype(np.float64) for q in p.psfs]
    gp, gk = O.poisson_nll_grad(psi, p.views, p.weights, psfs)
    r = rng(9)
    for _ in range(6):
        i = tuple(int(r.integers(0, s)) for s in psi.shape)
        a, b = psi.copy(), psi.copy()
        a[i] += 1e-4
        b[i] -= 1e-4
        fd = (O.poisson_nll(a, p.views, p.weights, psfs) - O.poisson_nll(b, p.views, p.weights, psfs)) / 2e-4
        assert gp[i] == pytest.approx(fd, rel=1e-4, abs=1e-6)
    for t in range(6):
        v = t % 2
        i = tuple(int(r.integers(0, s)) for s in psfs[v].shape)
        a = [q.copy() for q in psfs]
        b = [q.copy() for q in psfs]
        a[v][i] += 1e-5
        b[v][i] -= 1e-5
        fd = (O.poisson_nll(psi, p.views, p.weights, a) - O.poisson_nll(psi, p.views, p.weights, b)) / 2e-5
        assert gk[v][i] == pytest.approx(fd, rel=1e-4)


def test_transform_input_identity_and_shift():
    rng = np.random.default_rng(11)
    view = (rng.random((6, 7, 8)) * 10 + 1).astype(np.float32)
    eye = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    np.testing.assert_allclose(O.transform_input(view, eye, (0, 0, 0), view.shape), view, rtol=1e-12)
    # a registration shift of +2 in x moves the view to x >= 2 of the fused box; left of it is "no data"
    shifted = [1, 0, 0, 2, 0, 1, 0, 0, 0, 0, 1, 0]
    out = O.transform_input(view, shifted, (0, 0, 0), (6, 7, 10))
    np.testing.assert_allclose(out[:, :, 2:], view, rtol=1e-12)
    assert np.all(out[:, :, :2] == 0)


def test_blend_table_follows_the_reference_fill_loop():
    """BlendingRealRandomAccess fills its table by stepping d += 0.001 in double
    (BlendingRealRandomAccess.java:47-53): entry k holds the value at the accumulated d, whose
    last bits drift from k / 1000 (most doubles differ, no float does)."""
    lut = O._BLEND_LUT
    assert lut.shape == (1001,) and lut[0] == 0.0 and lut[1000] == 1.0
    exact = np.array([(math.cos((1 - k / 1000.0) * math.pi) + 1) / 2 for k in range(1001)])
    assert (lut != exact).sum() > 800
    np.testing.assert_array_equal(lut.astype(np.float32), exact.astype(np.float32))
    assert np.all(np.diff(lut) >= 0)


def test_transform_by_an_exact_quarter_turn_is_a_transpose():
    """A registration that turns the view by exactly 90 degrees about y (integer matrix) maps
    voxel centres onto voxel centres: the resampled view (TransformInput) and its blending weight
    are the view's own values and weights, transposed and flipped."""
    rng = np.random.default_rng(5)
    sz, sy, sx = 5, 6, 7
    view = (rng.random((sz, sy, sx)) * 10 + 1).astype(np.float32)
    # view -> world: x_w = z_v, y_w = y_v, z_w = (sx - 1) - x_v
    aff = [0, 0, 1, 0, 0, 1, 0, 0, -1, 0, 0, sx - 1]
    out = O.transform_input(view, aff, (0, 0, 0), (sx, sy, sz))
    want = np.transpose(view, (2, 1, 0))[::-1]  # out[z_w, y_w, x_w] = view[x_w, y_w, sx - 1 - z_w]
    np.testing.assert_array_equal(out, want)
    border, blend = (0.5, -2.0, 1.0), (3.0, 2.5, 2.0)
    w_turned = O.transform_weights(view.shape, aff, (0, 0, 0), (sx, sy, sz), border, blend)
    eye = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    w_view = O.transform_weights(view.shape, eye, (0, 0, 0), view.shape, border, blend)
    np.testing.assert_array_equal(w_turned, np.transpose(w_view, (2, 1, 0))[::-1])


def test_blending_weights_profile():
    # along x: 0 at the border, cosine ramp over `blending` voxels, 1 in the middle
    eye = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    w = O.transform_weights((9, 9, 41), eye, (0, 0, 0), (9, 9, 41), (0.0, -20.0, -20.0), (10.0, 1.0, 1.0))
    row = w[4, 4]
    assert row[0] == 0 and row[-1] == 0
    assert np.all(np.diff(row[:11]) >= 0) and np.all(row[10:31] == 1)
    np.testing.assert_allclose(row, row[::-1], atol=1e-6)
    assert row[5] == pytest.approx(0.5, abs=1e-6)


def test_virtual_weight_normalisation():
    rng = np.random.default_rng(12)
    ws = [rng.random((5, 6, 7)).astype(np.float32) * 0.9 for _ in range(4)]
    n1 = O.normalize_weights_virtual(ws, 1.0)
    s = np.sum(n1, axis=0)
    assert np.all(s <= 1 + 1e-6)
    big = np.sum(ws, axis=0) > 1
    np.testing.assert_allclose(s[big], 1, rtol=1e-5)
    np.testing.assert_allclose(n1[0][~big], ws[0][~big], rtol=1e-7)
    n2 = O.normalize_weights_virtual(ws, 3.0)
    assert np.all(n2[0] <= 1) and np.all(n2[0] >= np.minimum(1, n1[0] * 3 * (1 - 1e-6)))


def test_precomputed_weight_normalisation_and_overlap():
    rng = np.random.default_rng(13)
    ws = [np.where(rng.random((4, 5, 6)) < 0.3, 0, rng.random((4, 5, 6))).astype(np.float32) for _ in range(3)]
    ws[0][0, 0, 0] = ws[1][0, 0, 0] = ws[2][0, 0, 0] = 0  # no view: 0 / 0
    n = O.normalize_weights_precomputed(ws, 1.0)
    s = np.sum(n, axis=0)
    covered = np.sum(ws, axis=0) > 0
    assert np.all(np.isnan(s[~covered])) and not covered[0, 0, 0]
    np.testing.assert_allclose(s[covered], 1, rtol=1e-6)  # no guard: sums below 1 are raised too
    n2 = O.normalize_weights_precomputed(ws, 2.5)
    assert np.isnan(n2[0][0, 0, 0]) and np.nanmax(n2[0]) <= 1
    mn, avg = O.weight_overlap(ws, 7)
    cnt = sum((w > 0).astype(int) for w in ws).ravel()
    assert mn == 0
    # equal portions except the last one: the mean of portion means differs from the plain mean
    portions = O.divide_into_portions(cnt.size, 7)
    assert avg == pytest.approx(np.mean([cnt[s:s + l].mean() for s, l in portions]), rel=1e-12)


@pytest.mark.parametrize("cfg,psftype,lam", [(2, O.EFFICIENT_BAYESIAN, 0.006), (1, O.INDEPENDENT, 0.0),
                                             (2, O.OPTIMIZATION_I, 0.006)])
def test_fp64_torch_restatement_matches_the_numpy_oracle(cfg, psftype, lam):
    """The torch float64 restatement (the full-size checker) equals the numpy FP64 oracle on
    the CPU: same kernels, same first iteration, same updates, to rounding."""
    torch = pytest.importorskip("torch")
    from oracle import fp64_torch as T

    p = S.make_problem(cfg, shape_xyz=(30, 26, 22), psf_size_xyz=(7, 5, 9), n_blobs=8, iterations=2)
    want = O.Deconvolution(p.views, p.weights, p.psfs, psftype, lam, "f64", None)
    want.run(2)
    got = T.Deconvolution(p.views, p.weights, p.psfs, psftype, lam, device="cpu")
    got.run(2)
    assert got.avg == pytest.approx(want.avg, rel=1e-13)
    e = T.errors(torch.as_tensor(want.psi), got.psi)
    assert e["rel_l2"] < 1e-12, e
    for (_, _, s0, m0), (_, _, s1, m1) in zip(want.stats, got.stats):
        assert s1 == pytest.approx(s0, rel=1e-9) and m1 == pytest.approx(m0, rel=1e-9)
    np.testing.assert_allclose(got.masked_psi().numpy(), want.masked_psi(), rtol=1e-11, atol=1e-12)


def test_fp64_torch_convolution_matches_direct_convolution():
    torch = pytest.importorskip("torch")
    from oracle import fp64_torch as T

    r = rng(31)
    img = r.random((9, 11, 13))
    k = r.random((5, 3, 7))
    for mode, value in ((O.MIRROR, 0.0), (O.VALUE, 1.0)):
        c = T.Convolver(img.shape, k, "cpu")
        got = c(torch.as_tensor(img), mode, value).numpy()
        np.testing.assert_allclose(got, O.conv_direct(img, k, mode, value), rtol=1e-12, atol=1e-12)


def test_fp64_torch_nll_matches_the_numpy_oracle():
    pytest.importorskip("torch")
    from oracle import fp64_torch as T

    p = S.make_problem(5, shape_xyz=(20, 18, 16), psf_size_xyz=(5, 5, 7), n_blobs=10, n_views=2, iterations=1)
    psi = p.ground_truth.astype(np.float64) + 1.0
    want = O.poisson_nll(psi, p.views, p.weights, p.psfs)
    assert T.poisson_nll(psi, p.views, p.weights, p.psfs, device="cpu") == pytest.approx(want, rel=1e-12)


def test_simplex_projection():
    from spim_registration_gb300.psf_refine import project_simplex

    r = rng(41)
    for shape in ((7,), (3, 5, 7)):
        x = r.normal(size=shape) * 0.3
        p = project_simplex(x)
        assert p.shape == x.shape and np.all(p >= 0) and p.sum() == pytest.approx(1.0, abs=1e-12)
        # the projection is the closest simplex point: moving mass between two entries never helps
        for _ in range(50):
            i, j = r.integers(0, x.size, 2)
            t = min(1e-3, p.flat[i])
            q = p.copy()
            q.flat[i] -= t
            q.flat[j] += t
            assert np.sum((q - x) ** 2) >= np.sum((p - x) ** 2) - 1e-15
    y = np.abs(r.random(10))
    y /= y.sum()
    np.testing.assert_allclose(project_simplex(y), y, atol=1e-15)  # points of the simplex stay put
