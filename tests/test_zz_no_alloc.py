"""The allocation-free convolution entry point, mvd_convolve3d_device_noalloc (GPU).

Callers that may not call cudaMalloc / cudaFree while they run -- a streaming acquisition
pipeline that cannot take an allocation's device-wide synchronisation, or a host framework
whose memory manager owns the device pool -- use this variant.  It takes the same arguments
as mvd_convolve3d_device and works only inside the library's static device scratch.  This file
is collected last, so a run that stops at its first failure has run every other test already;
it passes both on its own in a fresh process and after the rest of the suite.
"""
import numpy as np
import pytest

from spim_registration_gb300 import native

pytestmark = pytest.mark.gpu

TOL = 2e-6  # the convolution tolerance of the other GPU tests (max abs error / max |value|)


def _case(torch, shape_zyx, kshape_zyx, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.rand(shape_zyx, device="cuda", generator=g) * 100
    k = torch.rand(kshape_zyx, device="cuda", generator=g)
    k /= k.sum()
    return x.contiguous(), k.contiguous()


def test_noalloc_matches_the_allocating_entry_point_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    lib = native.load()
    assert lib.getNumDevicesCUDA() >= 1
    cases = [((40, 48, 64), (25, 9, 9), 0, 0.0), ((17, 20, 33), (11, 7, 5), 1, 1.0)]
    for call, (shape, kshape, mode, value) in enumerate(cases):
        x, k = _case(torch, shape, kshape, seed=call)
        ref = torch.empty_like(x)
        got = torch.full_like(x, float("nan"))
        stream = torch.cuda.current_stream().cuda_stream
        dims = native.iarr([shape[2], shape[1], shape[0]])
        kd = native.iarr([kshape[2], kshape[1], kshape[0]])
        native.check(lib.mvd_convolve3d_device(x.data_ptr(), ref.data_ptr(), dims, k.data_ptr(), kd, mode, value, 0,
                                               stream))
        native.check(lib.mvd_convolve3d_device_noalloc(x.data_ptr(), got.data_ptr(), dims, k.data_ptr(), kd, mode,
                                                       value, 0, stream))
        torch.cuda.synchronize()
        r = ref.cpu().numpy().astype(np.float64)
        o = got.cpu().numpy().astype(np.float64)
        assert np.isfinite(o).all()
        assert np.abs(o - r).max() / np.abs(r).max() < TOL, call


def _noalloc(torch, lib, x, k, mode, value, stream):
    shape, kshape = tuple(x.shape), tuple(k.shape)
    got = torch.full_like(x, float("nan"))
    native.check(lib.mvd_convolve3d_device_noalloc(x.data_ptr(), got.data_ptr(),
                                                   native.iarr([shape[2], shape[1], shape[0]]), k.data_ptr(),
                                                   native.iarr([kshape[2], kshape[1], kshape[0]]), mode, value, 0,
                                                   stream))
    torch.cuda.synchronize()
    return got.cpu().numpy().astype(np.float64)


def test_noalloc_matches_the_fp64_oracle_for_both_extensions():
    """Checked against the CPU oracle directly, not only against the allocating entry point
    (a mistake both share in tile planning or in the gathers would pass that comparison)."""
    torch = pytest.importorskip("torch")
    from oracle import mvdecon_oracle as O

    lib = native.load()
    stream = torch.cuda.current_stream().cuda_stream
    cases = [((40, 48, 64), (25, 9, 9), O.MIRROR, 0.0), ((17, 20, 33), (11, 7, 5), O.VALUE, 1.0),
             ((31, 29, 37), (13, 5, 7), O.VALUE, 0.0), ((9, 50, 21), (3, 9, 9), O.MIRROR, 0.0)]
    for i, (shape, kshape, mode, value) in enumerate(cases):
        x, k = _case(torch, shape, kshape, seed=10 + i)
        want = O.conv_extended(x.cpu().numpy(), k.cpu().numpy(), mode, value)
        for call in range(2):  # the second call finds the array as the first one left it
            got = _noalloc(torch, lib, x, k, mode, value, stream)
            assert np.isfinite(got).all()
            assert np.abs(got - want).max() / np.abs(want).max() < TOL, (i, call)


def test_shared_memory_limits_stay_in_step_with_the_allocating_path():
    """An allocating call on a large volume, the allocation-free call on a small one, then an
    allocating call on a medium one: the kernels' shared-memory limits are raised through the
    same per-kernel record, so the third call still launches."""
    torch = pytest.importorskip("torch")
    from oracle import mvdecon_oracle as O

    lib = native.load()
    stream = torch.cuda.current_stream().cuda_stream

    def alloc(x, k, mode, value):
        out = torch.full_like(x, float("nan"))
        s, ks = tuple(x.shape), tuple(k.shape)
        native.check(lib.mvd_convolve3d_device(x.data_ptr(), out.data_ptr(), native.iarr([s[2], s[1], s[0]]),
                                               k.data_ptr(), native.iarr([ks[2], ks[1], ks[0]]), mode, value, 0,
                                               stream))
        torch.cuda.synchronize()
        return out.cpu().numpy().astype(np.float64)

    big = _case(torch, (64, 160, 200), (21, 9, 9), seed=21)
    small = _case(torch, (12, 16, 20), (5, 3, 3), seed=22)
    medium = _case(torch, (48, 120, 150), (15, 7, 7), seed=23)
    for (x, k), fn in ((big, alloc), (small, lambda x, k, m, v: _noalloc(torch, lib, x, k, m, v, stream)),
                       (medium, alloc)):
        want = O.conv_extended(x.cpu().numpy(), k.cpu().numpy(), O.MIRROR)
        got = fn(x, k, 0, 0.0)
        assert np.abs(got - want).max() / np.abs(want).max() < TOL


def test_noalloc_refuses_a_capturing_stream():
    torch = pytest.importorskip("torch")
    lib = native.load()
    x, k = _case(torch, (12, 16, 20), (5, 3, 3), seed=5)
    out = torch.empty_like(x)
    _noalloc(torch, lib, x, k, 0, 0.0, torch.cuda.current_stream().cuda_stream)  # set-up outside the capture
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    st = None
    with torch.cuda.stream(s):
        g.capture_begin()
        try:
            st = lib.mvd_convolve3d_device_noalloc(x.data_ptr(), out.data_ptr(), native.iarr([20, 16, 12]),
                                                   k.data_ptr(), native.iarr([3, 3, 5]), 0, 0.0, 0, s.cuda_stream)
        finally:
            g.capture_end()
    assert st == 4  # MVD_ERR_STATE
    assert "captured" in lib.mvd_last_error().decode()


def test_noalloc_rejects_volumes_beyond_its_scratch():
    pytest.importorskip("torch")
    lib = native.load()
    dims = native.iarr([512, 512, 256])
    kd = native.iarr([31, 31, 61])
    st = lib.mvd_convolve3d_device_noalloc(None, None, dims, None, kd, 0, 0.0, 0, None)
    assert st == 1  # NULL pointers are rejected before anything else
    import torch

    x = torch.zeros(8, device="cuda")
    st = lib.mvd_convolve3d_device_noalloc(x.data_ptr(), x.data_ptr(), dims, x.data_ptr(), kd, 0, 0.0, 0, None)
    assert st == 1
    assert "bytes of scratch" in lib.mvd_last_error().decode()
