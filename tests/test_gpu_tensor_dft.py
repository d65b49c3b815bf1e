"""The z pass with its middle 16-point DFTs on the tensor cores (MVD_FLAG_TENSOR_DFT, GPU).

The pencils of the 512x512x256 workload are 320 = 20 x 16 and 288 = 18 x 16 long; with the flag
their forward and inverse 16-point DFTs run as TF32 products on tcgen05 with a three-term hi/lo
split and FP32 accumulation.  The method's gate is the same as for the FP32 SIMT path: relative
L2 <= 1e-4 against the FP64 oracle after 10 iterations (MVDeconvolution.java:354-465); max-abs is
reported, and the result must stay close to the SIMT path's.
"""
import numpy as np
import pytest

from spim_registration_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

GATE = 1e-4


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def _run(prob, flags, iterations):
    from spim_registration_gb300 import Deconvolution

    with Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, 0, flags) as d:
        d.run(iterations)
        d.synchronize()  # reports a tensor-core stage whose bounded wait gave up
        plans = [d.plan(v) for v in range(len(prob.views))]
        return d.get_psi(), plans


@pytest.mark.parametrize("shape", [(260, 260, 256), (512, 512, 256)])
def test_tensor_core_stages_match_fp64(torch, shape):
    from oracle import fp64_torch as T
    from spim_registration_gb300 import FLAG_AUTOTUNE, FLAG_TENSOR_DFT

    prob = S.make_problem(4, shape_xyz=shape, psf_size_xyz=(31, 31, 61), n_blobs=None if shape[0] == 512 else 400)
    flags = FLAG_TENSOR_DFT | (FLAG_AUTOTUNE if shape[0] == 512 else 0)
    got, plans = _run(prob, flags, 10)
    assert any(p["tensor_dft"] for p in plans), plans  # pencils with a tensor-core z pass
    simt, _ = _run(prob, flags & ~FLAG_TENSOR_DFT, 10)
    ref = T.Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, device="cuda:0")
    ref.run(10)
    e = T.errors(got, ref.psi)
    es = T.errors(simt, ref.psi)
    print(f"{shape}: tensor-core relL2 {e['rel_l2']:.3e} max-abs {e['max_abs']:.3e}; "
          f"SIMT relL2 {es['rel_l2']:.3e} max-abs {es['max_abs']:.3e}; plans {[p['tile'] for p in plans]}")
    assert e["rel_l2"] <= GATE, e
    assert np.linalg.norm(got - simt) / np.linalg.norm(simt) < 1e-5


SCRIPT = """
import sys
import numpy as np
sys.path.insert(0, {root!r})
from spim_registration_gb300 import FLAG_TENSOR_DFT, Deconvolution, native
from spim_registration_gb300 import synthetic as S
p = S.make_problem(4, shape_xyz=(200, 120, 256), psf_size_xyz=(31, 31, 61), n_blobs=40, iterations=1)
with Deconvolution(p.views, p.weights, p.psfs, p.psftype, p.lam, 0, FLAG_TENSOR_DFT) as d:
    d.run(1)
    try:
        d.synchronize()
        print("no error")
    except native.MvdError as e:
        print("error:", e)
# the context is still usable: the default path runs and its result is finite
with Deconvolution(p.views, p.weights, p.psfs, p.psftype, p.lam, 0, 0) as d:
    d.run(1)
    d.synchronize()
    print("finite", bool(np.isfinite(d.get_psi()).all()))
"""


def test_a_wait_that_runs_out_is_reported_and_the_context_stays_usable():
    """MVD_TC_WAIT_POLLS=0: every MMA wait of the tensor-core z pass gives up at once.  Each CTA
    counts the failure, waits (bounded) for its products in flight, frees its tensor memory and
    returns; mvd_synchronize reports the count, and later work in the same process runs."""
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, MVD_TC_WAIT_POLLS="0")
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=root)], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "gave up waiting" in r.stdout, r.stdout
    assert "finite True" in r.stdout, r.stdout
