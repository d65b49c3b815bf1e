"""The compile-time-shaped plane kernels against the generic ones (GPU).

A cfg2-shaped problem (4 views, 172 x 172 x 192, rotated 15 x 15 x 41 PSFs) plans compiled tile
shapes and pencil lengths;
the same deconvolution in a child process with MVD_FIXED_PLANES=0 runs the generic kernels.
Both use the same radices, twiddles and functors, so psi must agree bit for bit."""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = textwrap.dedent("""
    import sys
    import numpy as np
    sys.path.insert(0, {root!r})
    from spim_registration_gb300 import Deconvolution
    from spim_registration_gb300 import synthetic as S
    p = S.make_problem(2, shape_xyz=(172, 172, 192), psf_size_xyz=(15, 15, 41), n_blobs=40, iterations=2)
    d = Deconvolution(p.views, p.weights, p.psfs, p.psftype, p.lam)
    d.run(2)
    np.save(sys.argv[1], d.get_psi())
    print(" ".join("%dx%dx%d" % tuple(d.plan(v)["tile"]) for v in range(len(p.views))))
""")


def _run(out, fixed):
    env = dict(os.environ, MVD_FIXED_PLANES="1" if fixed else "0")
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT), out], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout.split()


def test_fixed_shape_kernels_equal_the_generic_kernels(tmp_path):
    a, b = str(tmp_path / "fixed.npy"), str(tmp_path / "generic.npy")
    shapes = _run(a, True)
    assert _run(b, False) == shapes
    assert any(t.startswith("100x100x") for t in shapes)  # a compiled plane shape was planned
    assert any(t.endswith("x240") or t.endswith("x216") for t in shapes)  # and a compiled pencil length
    np.testing.assert_array_equal(np.load(a), np.load(b))
