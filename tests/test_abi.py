"""The C-ABI library builds, loads and exports every symbol include/mvdecon.h declares (no GPU)."""
import ctypes
import os

import pytest

from spim_registration_gb300 import _build, native


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_build.library_path()):
        _build.build()
    return native.load()


def test_exports_every_declared_symbol(lib):
    names = native.header_symbols()
    assert "convolution3DfftCUDAInPlace" in names and "mvd_create" in names
    raw = ctypes.CDLL(_build.library_path())
    for n in names:
        assert hasattr(raw, n), n
        assert n in native.SIGNATURES, n


def test_jna_names_of_the_reference_interfaces(lib):
    # CUDAStandardFunctions.java:36-44 and CUDAFourierConvolution.java:30-31
    for n in ["getCUDAcomputeCapabilityMinorVersion", "getCUDAcomputeCapabilityMajorVersion", "getNumDevicesCUDA",
              "getNameDeviceCUDA", "getMemDeviceCUDA", "getFreeMemDeviceCUDA", "convolution3DfftCUDA",
              "convolution3DfftCUDAInPlace"]:
        assert hasattr(lib, n)


def test_aliases_point_to_the_library(lib):
    for name in _build.ALIASES:
        alias = os.path.join(_build.LIBDIR, name)
        assert os.path.realpath(alias) == os.path.realpath(_build.library_path())
    # the detection plugin loads the separable library by a name containing "separable"
    # (DifferenceOfGaussian.java:366-369)
    assert any("separable" in n.lower() for n in _build.ALIASES)


def test_jna_names_of_the_separable_interface(lib):
    # CUDASeparableConvolution.java:34-46
    for n in ["convolve_127", "convolve_63", "convolve_31", "convolve_15", "convolve_7", "convolutionCPU"]:
        assert hasattr(lib, n)


def test_device_count_semantics(lib):
    n = lib.getNumDevicesCUDA()
    assert n == -1 or n >= 0  # -1 = driver failure (CUDAStandardFunctions.java:38-41)


def test_version_string(lib):
    assert b"sm_103a" in lib.mvd_version()
