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
    if sys.argv[2] == "large":  # the 512x512x256 workload's PSFs: 160x160 / 192x96 planes, 320 / 288 pencils
        p = S.make_problem(4, shape_xyz=(260, 260, 256), psf_size_xyz=(31, 31, 61), n_blobs=60, iterations=1)
    elif sys.argv[2] == "large135":  # 192x135 planes (radices 15 x 9 along y)
        p = S.make_problem(4, shape_xyz=(248, 210, 256), psf_size_xyz=(31, 31, 61), n_blobs=60, iterations=1)
    elif sys.argv[2] == "full":
        p = S.make_problem(2, shape_xyz=(172, 172, 192), psf_size_xyz=(15, 15, 41), n_blobs=40, iterations=2)
    else:  # data boxes smaller than the volume in x, y and z, still planned with 100/128-wide tiles
        p = S.make_problem(2, shape_xyz=(256, 256, 24), psf_size_xyz=(15, 15, 41), n_blobs=40, iterations=2)
        for img, w in zip(p.views, p.weights):
            for a in (img, w):
                a[:, :, :3] = 0; a[:, :, 253:] = 0; a[:, :2, :] = 0; a[:, 254:, :] = 0; a[20:, :, :] = 0
    d = Deconvolution(p.views, p.weights, p.psfs, p.psftype, p.lam)
    d.run(2)
    np.save(sys.argv[1], d.get_psi())
    print(" ".join("%dx%dx%d" % tuple(d.plan(v)["tile"]) for v in range(len(p.views))))
""")


def _run(out, fixed, case="full", cap=None, staged=False, z_in_place=True):
    env = dict(os.environ, MVD_FIXED_PLANES="1" if fixed else "0", MVD_STAGED_PLANES="1" if staged else "0",
               MVD_Z_INPLACE="1" if z_in_place else "0")
    if cap:
        env["MVD_PLANE_CAP"] = str(cap)
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT), out, case], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout.split()


def test_fixed_shape_kernels_equal_the_generic_kernels(tmp_path):
    a, b = str(tmp_path / "fixed.npy"), str(tmp_path / "generic.npy")
    shapes = _run(a, True)
    assert _run(b, False) == shapes
    assert any(t.startswith("100x100x") for t in shapes)  # a compiled plane shape was planned
    assert any(t.endswith("x240") or t.endswith("x216") for t in shapes)  # and a compiled pencil length
    np.testing.assert_array_equal(np.load(a), np.load(b))


@pytest.mark.parametrize("cap,plane,case", [(14336, "160x160x", "large"), (10240, "192x96x", "large"),
                                            (14336, "192x135x", "large135")])
def test_large_psf_shapes_equal_the_generic_kernels(tmp_path, cap, plane, case):
    """1024-thread compiled planes (plain row layout) and the 320 / 288 compiled pencils (radices
    20 and 18) of the 31x31x61-PSF workload against the generic kernels, bit for bit."""
    a, b = str(tmp_path / "fixed.npy"), str(tmp_path / "generic.npy")
    shapes = _run(a, True, case, cap)
    assert _run(b, False, case, cap) == shapes
    assert any(t.startswith(plane) for t in shapes), shapes
    assert any(t.endswith("x320") for t in shapes) and (cap == 14336 or any(t.endswith("x288") for t in shapes))
    np.testing.assert_array_equal(np.load(a), np.load(b))


@pytest.mark.parametrize("cap,plane,case", [(14336, "160x160x", "large"), (10240, "192x96x", "large"),
                                            (14336, "192x135x", "large135")])
def test_in_place_plane_kernels_equal_the_two_buffer_kernels(tmp_path, cap, plane, case):
    """The in-place plane kernels (one shared buffer, stages staged through tensor memory, two
    CTAs per SM) against the two-buffer compiled kernels, bit for bit."""
    a, b = str(tmp_path / "staged.npy"), str(tmp_path / "two_buffer.npy")
    shapes = _run(a, True, case, cap, staged=True)
    assert _run(b, True, case, cap, staged=False) == shapes
    assert any(t.startswith(plane) for t in shapes), shapes
    np.testing.assert_array_equal(np.load(a), np.load(b))


@pytest.mark.parametrize("case,lengths", [("full", ("x240", "x216")), ("large", ("x320", "x288"))])
def test_in_place_z_pass_equals_the_two_buffer_z_pass(tmp_path, case, lengths):
    """The one-buffer z pass (middle stage written back in place, four CTAs per SM) against the
    two-buffer compiled z pass, bit for bit, on the compiled pencil lengths of both workloads."""
    a, b = str(tmp_path / "in_place.npy"), str(tmp_path / "two_buffer.npy")
    cap = 10240 if case == "large" else None
    shapes = _run(a, True, case, cap, staged=True)
    assert _run(b, True, case, cap, staged=True, z_in_place=False) == shapes
    assert any(t.endswith(lengths) for t in shapes), shapes
    np.testing.assert_array_equal(np.load(a), np.load(b))
