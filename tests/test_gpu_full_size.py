"""Parity at the benchmark's own sizes and plans (GPU).

The other GPU tests run volumes small enough for the numpy oracle.  Here the 4-view
512x512x256 workload (PSF 31x31x61, rotated views with 65x31x65 PSFs) and the 4-view
256x256x192 workload (PSF 15x15x41) run at full size with the autotuned tile plans that
bench.py times, and the plain FP32 form with the reference's block structure, each against
the oracle's float64 deconvolution (its torch restatement, pinned to the numpy oracle in
tests/test_oracle.py).  The method's gate is relative L2 <= 1e-4 after 10 iterations
(MVDeconvolution.java:354-465, MVDeconFFT.java:384-560); max-abs is reported.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GATE = 1e-4


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


_problems = {}


def _problem(cfg):
    from spim_registration_gb300 import synthetic as S

    if cfg not in _problems:
        shape, psf = {2: ((256, 256, 192), (15, 15, 41)), 4: ((512, 512, 256), (31, 31, 61)),
                      3: ((256, 256, 256), (15, 15, 41))}[cfg]
        _problems[cfg] = S.make_problem(cfg, shape_xyz=shape, psf_size_xyz=psf)
    return _problems[cfg]


def _check(torch, dec, prob, iterations, label):
    from oracle import fp64_torch as T

    dec.run(iterations)
    got = dec.get_psi()
    ref = T.Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, device="cuda:0")
    ref.run(iterations)
    e = T.errors(got, ref.psi)
    plans = [dec.plan(v) for v in range(len(prob.views))]
    print(f"{label}: relL2 {e['rel_l2']:.3e} max-abs {e['max_abs']:.3e} ({e['max_abs_rel']:.2e} of max); "
          f"plans {[(p['tiles'], p['tile']) for p in plans]}")
    del ref
    torch.cuda.empty_cache()
    assert e["rel_l2"] <= GATE, (label, e)
    return e


@pytest.mark.parametrize("cfg", [4, 2])
def test_autotuned_plans_at_full_size_match_fp64(torch, cfg):
    from spim_registration_gb300 import FLAG_AUTOTUNE, Deconvolution

    prob = _problem(cfg)
    with Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, 0, FLAG_AUTOTUNE) as dec:
        _check(torch, dec, prob, 10, f"cfg{cfg} autotuned")


@pytest.mark.parametrize("cfg", [4, 2])
def test_default_plans_at_full_size_match_fp64(torch, cfg):
    from spim_registration_gb300 import Deconvolution

    prob = _problem(cfg)
    with Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, 0, 0) as dec:
        _check(torch, dec, prob, 10, f"cfg{cfg} default plans")


@pytest.mark.parametrize("cfg,block", [(4, None), (2, (128, 128, 128))])
def test_plain_form_at_full_size_matches_fp64(torch, cfg, block):
    """The plain form (the bench's denominator) on the same inputs, 2 iterations: every block's
    effective region is exact linear convolution, so the blocked result equals the whole-image
    one."""
    from spim_registration_gb300 import FLAG_PLAIN, Deconvolution

    prob = _problem(cfg)
    with Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, 0, FLAG_PLAIN, block) as dec:
        e = _check(torch, dec, prob, 2, f"cfg{cfg} plain form")
    assert e["max_abs_rel"] < 1e-4


def test_cropped_views_at_full_size_match_fp64(torch):
    """Six views cropped to random boxes in a 256^3 volume: each view's tiles cover its own data
    box (uneven tile grids), autotuned."""
    from spim_registration_gb300 import FLAG_AUTOTUNE, Deconvolution

    prob = _problem(3)
    with Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, 0, FLAG_AUTOTUNE) as dec:
        _check(torch, dec, prob, 10, "cfg3 autotuned")
