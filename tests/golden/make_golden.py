"""Writes the golden fixtures of tests/golden/ from the CPU oracle (oracle/mvdecon_oracle.py).

The reference ships no golden data for this path, so these fixtures pin the oracle's own
results on small seeded inputs: the CPU tests check that the oracle still reproduces them and
the GPU tests check the library against them.  Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import mvdecon_oracle as O  # noqa: E402
from spim_registration_gb300 import synthetic as S  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def conv_fixture():
    rng = np.random.default_rng(7)
    img = (rng.random((12, 14, 16)) * 100).astype(np.float32)
    k = rng.random((7, 3, 5)).astype(np.float32)
    k /= k.sum()
    return dict(img=img, kernel=k, mirror=O.conv_extended(img, k, O.MIRROR, 0.0, "f64"),
                value1=O.conv_extended(img, k, O.VALUE, 1.0, "f64"))


def decon_fixture(cfg, shape, psf, iterations, n_views=None, psftype=None):
    p = S.make_problem(cfg, shape_xyz=shape, psf_size_xyz=psf, n_blobs=12, iterations=iterations,
                       n_views=n_views, psftype=psftype)
    psi, d = O.deconvolve(p, arith="f64", block=None, mask=False)
    out = dict(psi=psi, avg=np.float64(d.avg), psftype=np.int32(p.psftype), lam=np.float64(p.lam),
               iterations=np.int32(p.iterations), nviews=np.int32(len(p.views)))
    for i in range(len(p.views)):
        out[f"view{i}"], out[f"weight{i}"], out[f"psf{i}"] = p.views[i], p.weights[i], p.psfs[i]
        out[f"k2_{i}"] = d.k2[i]
    return out


def main():
    np.savez_compressed(os.path.join(HERE, "conv_12x14x16_k5x3x7.npz"), **conv_fixture())
    np.savez_compressed(os.path.join(HERE, "decon_cfg1_32x24x16.npz"), **decon_fixture(1, (32, 24, 16), (5, 5, 9), 3))
    np.savez_compressed(os.path.join(HERE, "decon_cfg2_eb_24x24x20.npz"),
                        **decon_fixture(2, (24, 24, 20), (5, 5, 9), 2, n_views=3))
    print("written to", HERE)


if __name__ == "__main__":
    main()
