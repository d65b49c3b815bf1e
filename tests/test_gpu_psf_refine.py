"""PSF refinement from bead data at a realistic PSF size (GPU).

Two views of 96^3 with 120 point-like beads (sigma 0.7, peak U[500, 2000]) and the 31x31x61
PSF (sigma 2, 2, 7) rotated per view (31x31x61 and, at 45 degrees, 65x31x65): the starting PSFs are 20% too
wide.  At this size the tiles' windows and the PSF halos interact (every tile is mostly halo),
and each view's blur is recomputed tile by tile inside mvd_backward.  Checked:

* the PSF gradient and the estimate gradient against FP64 central finite differences of the
  oracle's NLL (its float64 restatement on the GPU) at 64 random voxels, relative error <= 1e-3;
* projected gradient refinement: the NLL never increases, the PSFs stay non-negative with unit
  sum, and they move towards the true PSFs.
"""
import numpy as np
import pytest

from spim_registration_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

SIGMA = (2.0, 2.0, 7.0)
PSF = (31, 31, 61)
ANGLES = (0, 45)  # the first two views of the bead configuration


@pytest.fixture(scope="module")
def beads():
    p = S.make_problem(5, shape_xyz=(96, 96, 96), psf_size_xyz=PSF, n_blobs=120, n_views=2, iterations=1)
    wide = [S.gaussian_psf(tuple(1.2 * s for s in SIGMA), PSF, a) for a in ANGLES]
    true = [(q / q.sum()).astype(np.float64) for q in p.psfs]
    psi = p.ground_truth.astype(np.float32)
    return p, wide, true, psi


def _nll_terms(torch, psi, views, weights, psfs):
    """Per-voxel NLL terms of every view in float64 on the GPU (the oracle's NLL before its
    final sum), so that finite differences subtract voxel by voxel."""
    from oracle import fp64_torch as T
    from oracle import mvdecon_oracle as O

    p = torch.as_tensor(np.asarray(psi, dtype=np.float64), device="cuda")
    out = []
    for img, w, k in zip(views, weights, psfs):
        f = T.Convolver(p.shape, np.asarray(k, dtype=np.float64), "cuda")(p, O.MIRROR)
        im = torch.as_tensor(img, device="cuda").double()
        wt = torch.as_tensor(w, device="cuda").double()
        m = im > 0
        out.append(torch.where(m, wt * (f - im * torch.log(torch.where(m, f, torch.ones_like(f)))),
                               torch.zeros_like(f)))
    return out


def _fd(torch, a_terms, b_terms, step):
    return sum(float((a - b).sum().item()) for a, b in zip(a_terms, b_terms)) / (2 * step)


def test_gradients_match_fp64_finite_differences_at_psf_31x31x61(beads):
    torch = pytest.importorskip("torch")
    from spim_registration_gb300.psf_refine import PSFRefinement

    p, wide, _, psi = beads
    with PSFRefinement(p.views, p.weights, wide, psi) as r:
        k = [x.copy() for x in r.psfs]
        g_psi, g_psf = r.dec.backward()
    psi64 = psi.astype(np.float64)
    rng = np.random.default_rng(7)
    psi_scale = np.sqrt(np.mean(g_psi.astype(np.float64) ** 2))
    errs = []
    for _ in range(32):  # estimate voxels
        i = tuple(int(rng.integers(0, s)) for s in psi.shape)
        eps = 1e-2 * max(psi64[i], 1.0)
        a, b = psi64.copy(), psi64.copy()
        a[i] += eps
        b[i] -= eps
        fd = _fd(torch, _nll_terms(torch, a, p.views, p.weights, k), _nll_terms(torch, b, p.views, p.weights, k), eps)
        errs.append(abs(g_psi[i] - fd) / max(abs(fd), 1e-2 * psi_scale))
    for t in range(32):  # PSF voxels, inside the support where the PSF is not negligible
        v = t % len(k)
        big = np.argwhere(k[v] > 1e-3 * k[v].max())
        i = tuple(int(c) for c in big[rng.integers(0, len(big))])
        h = 1e-3 * k[v][i]
        a = [x.copy() for x in k]
        b = [x.copy() for x in k]
        a[v][i] += h
        b[v][i] -= h
        fd = _fd(torch, _nll_terms(torch, psi64, p.views, p.weights, a),
                 _nll_terms(torch, psi64, p.views, p.weights, b), h)
        scale = np.sqrt(np.mean(g_psf[v].astype(np.float64) ** 2))
        errs.append(abs(g_psf[v][i] - fd) / max(abs(fd), 1e-2 * scale))
    assert max(errs) <= 1e-3, (max(errs), int(np.argmax(errs)))


def test_projected_gradient_refinement_moves_towards_the_true_psf(beads):
    pytest.importorskip("torch")
    from spim_registration_gb300.psf_refine import PSFRefinement

    p, wide, true, psi = beads
    with PSFRefinement(p.views, p.weights, wide, psi) as r:
        start = [float(np.linalg.norm(q - t) / np.linalg.norm(t)) for q, t in zip(r.psfs, true)]
        r.run(12)
        nll = [h.nll for h in r.history]
        end = [float(np.linalg.norm(q - t) / np.linalg.norm(t)) for q, t in zip(r.psfs, true)]
        for q in r.psfs:
            assert q.min() >= 0 and q.sum() == pytest.approx(1.0, abs=1e-9)
    print(f"NLL {nll[0]:.6e} -> {nll[-1]:.6e}; PSF rel. L2 to the truth {start} -> {end}")
    assert all(b <= a for a, b in zip(nll, nll[1:]))
    assert nll[-1] < nll[0]
    assert all(e < 0.7 * s for s, e in zip(start, end))
