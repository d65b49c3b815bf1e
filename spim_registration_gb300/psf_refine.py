"""PSF refinement from bead data through the forward/backward pair of the image-formation model.

The reference builds each view's PSF from its bead detections and never changes it afterwards
(``ExtractPSF.extractPSFLocal`` / ``transformPSF``, ExtractPSF.java:277-464).  A PSF that is too
wide (a poor bead fit, a defocused bead image) then limits every deconvolution that uses it.
Here the PSFs are refined against the multiview Poisson model of the views themselves:

    NLL(P) = sum_v sum_{img_v > 0} w_v (f_v - img_v log f_v),   f_v = ext(psi) (*) P_v,

with psi the bead image (the calibration object: point-like beads at their fitted positions
and amplitudes).  ``mvd_forward`` evaluates NLL and ``mvd_backward`` its gradient with
respect to every PSF voxel (recomputing each view's blur tile by tile); each step is a
projected gradient step per view,

    P_v <- Proj( P_v - eta_v dNLL/dP_v ),   Proj = Euclidean projection onto
           { P >= 0, sum P = 1 }  (positivity and the unit sum of AdjustInput.normImg,
           AdjustInput.java:50-56),

with a backtracking step size that guarantees the NLL never increases.  The refined kernel is
installed with ``mvd_set_kernel`` (its spectrum is rebuilt on the GPU).
"""
from __future__ import annotations

import dataclasses

import numpy as np

from .mvdecon import PSFTYPE, Deconvolution


def project_simplex(p: np.ndarray) -> np.ndarray:
    """Euclidean projection of ``p`` onto the probability simplex {x >= 0, sum x = 1}: the
    sort-based method of Duchi, Shalev-Shwartz, Singer and Chandra ("Efficient projections onto
    the l1-ball for learning in high dimensions", ICML 2008).  Computed in float64."""
    v = np.asarray(p, dtype=np.float64).ravel()
    u = np.sort(v)[::-1]
    css = np.cumsum(u) - 1.0
    j = np.arange(1, v.size + 1)
    rho = int(np.nonzero(u - css / j > 0)[0][-1])
    theta = css[rho] / (rho + 1)
    return np.maximum(v - theta, 0.0).reshape(np.shape(p))


@dataclasses.dataclass
class RefineStep:
    step: int
    nll: float
    step_sizes: list
    backtracks: int


class PSFRefinement:
    """Projected-gradient refinement of every view's PSF at a fixed estimate psi.

    ``views``/``weights`` are the observed views and their weights ([z, y, x] float32);
    ``psfs`` the starting PSFs (odd sizes; normalised to unit sum on upload); ``psi`` the bead
    image the views are modelled from."""

    def __init__(self, views, weights, psfs, psi, device: int = 0):
        # the kernel preparation of INDEPENDENT is the cheapest; forward/backward use kernel1 only
        self.dec = Deconvolution(views, weights, psfs, PSFTYPE.INDEPENDENT, 0.0, device)
        self.dec.set_psi(np.ascontiguousarray(psi, dtype=np.float32))
        self.n_views = len(psfs)
        self.psfs = [self.dec.kernel(v, 1).astype(np.float64) for v in range(self.n_views)]
        self.eta = [None] * self.n_views
        self.nll = self.dec.forward()
        self.history = [RefineStep(0, self.nll, [0.0] * self.n_views, 0)]

    def close(self):
        self.dec.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def _install(self, v, p):
        self.dec.set_kernel(v, 1, p.astype(np.float32))

    def step(self, max_backtracks: int = 12) -> RefineStep:
        """One projected gradient step on every view's PSF (views in turn, each with its own
        backtracking search on the sufficient-decrease condition of projected gradient descent:
        NLL(P+) <= NLL(P) + g.(P+ - P) + |P+ - P|^2 / (2 eta))."""
        _, grads = self.dec.backward()
        backtracks = 0
        for v in range(self.n_views):
            g = grads[v].astype(np.float64)
            p = self.psfs[v]
            if self.eta[v] is None:  # first step: move about 10% of the PSF's norm
                self.eta[v] = 0.1 * np.linalg.norm(p) / max(np.linalg.norm(g), 1e-300)
            eta = self.eta[v] * 2.0
            accepted = False
            for _ in range(max_backtracks):
                cand = project_simplex(p - eta * g)
                d = cand - p
                self._install(v, cand)
                nll = self.dec.forward()
                if nll <= self.nll + float(np.sum(g * d)) + float(np.sum(d * d)) / (2.0 * eta) and nll <= self.nll:
                    accepted = True
                    break
                eta *= 0.5
                backtracks += 1
            if accepted:
                self.psfs[v] = cand
                self.nll = nll
                self.eta[v] = eta
            else:
                self._install(v, p)  # no decrease found: keep the PSF
                self.eta[v] = eta
        rec = RefineStep(len(self.history), self.nll, list(self.eta), backtracks)
        self.history.append(rec)
        return rec

    def run(self, steps: int):
        for _ in range(steps):
            self.step()
        return self.psfs


def refine_psfs(views, weights, psfs, psi, steps: int = 20, device: int = 0):
    """Refined PSFs (float32, unit sum) and the NLL after every step."""
    with PSFRefinement(views, weights, psfs, psi, device) as r:
        r.run(steps)
        return [p.astype(np.float32) for p in r.psfs], [h.nll for h in r.history]
