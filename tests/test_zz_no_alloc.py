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
