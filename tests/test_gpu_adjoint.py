"""Forward/backward pair of the multiview Poisson image-formation model (GPU).

NLL(psi, P) = sum_v sum_{img_v > 0} w_v (f_v - img_v log f_v),  f_v = ext(psi) (*) P_v.
The library's mvd_forward / mvd_backward are checked against the oracle's analytic FP64
gradient and against FP64 central finite differences of the oracle's NLL at 64 random voxels
(psi voxels and PSF voxels), relative error <= 1e-3.
"""
import numpy as np
import pytest

from oracle import mvdecon_oracle as O
from spim_registration_gb300 import Deconvolution
from spim_registration_gb300 import synthetic as S
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    # config 5 in miniature: beads (sigma 0.7, peak U[500, 2000]), rotated PSFs, blended weights
    p = S.make_problem(5, shape_xyz=(36, 32, 28), psf_size_xyz=(7, 7, 11), n_blobs=40, n_views=3, iterations=2)
    d = Deconvolution(p.views, p.weights, p.psfs, p.psftype, p.lam)
    d.run(2)  # a psi away from the flat start
    psi = d.get_psi().astype(np.float64)
    k1 = [d.kernel(v, 1).astype(np.float64) for v in range(len(p.psfs))]
    return p, d, psi, k1


def test_forward_matches_oracle_nll(case):
    p, d, psi, k1 = case
    want = O.poisson_nll(psi, p.views, p.weights, k1)
    got = d.forward()
    assert got == pytest.approx(want, rel=2e-5)


def test_backward_matches_oracle_gradient(case):
    p, d, psi, k1 = case
    g_psi, g_psf = d.backward()
    w_psi, w_psf = O.poisson_nll_grad(psi, p.views, p.weights, k1)
    assert rel_l2(g_psi, w_psi) < 1e-4
    for a, b in zip(g_psf, w_psf):
        assert rel_l2(a, b) < 1e-4


def test_backward_matches_fp64_finite_differences(case):
    p, d, psi, k1 = case
    g_psi, g_psf = d.backward()
    rng = np.random.default_rng(5)
    eps = 1e-3
    psi_scale = np.sqrt(np.mean(g_psi.astype(np.float64) ** 2))
    errs = []
    for _ in range(32):  # psi voxels
        i = tuple(int(rng.integers(0, s)) for s in psi.shape)
        a, b = psi.copy(), psi.copy()
        a[i] += eps
        b[i] -= eps
        fd = (O.poisson_nll(a, p.views, p.weights, k1) - O.poisson_nll(b, p.views, p.weights, k1)) / (2 * eps)
        errs.append(abs(g_psi[i] - fd) / max(abs(fd), 1e-2 * psi_scale))
    for t in range(32):  # PSF voxels
        v = t % len(k1)
        i = tuple(int(rng.integers(0, s)) for s in k1[v].shape)
        h = 1e-6
        a = [k.copy() for k in k1]
        b = [k.copy() for k in k1]
        a[v][i] += h
        b[v][i] -= h
        fd = (O.poisson_nll(psi, p.views, p.weights, a) - O.poisson_nll(psi, p.views, p.weights, b)) / (2 * h)
        scale = np.sqrt(np.mean(g_psf[v].astype(np.float64) ** 2))
        errs.append(abs(g_psf[v][i] - fd) / max(abs(fd), 1e-2 * scale))
    assert max(errs) <= 1e-3, max(errs)


def test_set_kernel_changes_the_model(case):
    p, d, psi, k1 = case
    base = d.forward()
    wider = S.gaussian_psf((1.6, 1.6, 4.0), (7, 7, 11), 0.0)
    wider = (wider / wider.sum()).astype(np.float32)
    old = d.kernel(0, 1)
    d.set_kernel(0, 1, wider)
    k = [wider.astype(np.float64)] + k1[1:]
    assert d.forward() == pytest.approx(O.poisson_nll(psi, p.views, p.weights, k), rel=2e-5)
    d.set_kernel(0, 1, old)
    assert d.forward() == pytest.approx(base, rel=1e-6)
