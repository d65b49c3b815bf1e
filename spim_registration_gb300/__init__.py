"""GB300-native multiview Bayesian deconvolution (fiji/SPIM_Registration hot path).

The compute path is ``lib/libFourierConvolutionCUDA.so`` (sm_103a CUDA, C ABI in
``include/mvdecon.h``); this package holds its build step, the ctypes binding and the
Python mirror of the reference's Java classes.
"""
from .mvdecon import (  # noqa: F401
    FLAG_AUTOTUNE,
    FLAG_NO_GRAPH,
    FLAG_PLAIN,
    FLAG_REF_SUM_THREADS,
    FLAG_TENSOR_DFT,
    PSFTYPE,
    CUDAFourierConvolution,
    Deconvolution,
    MVDeconFFT,
    MVDeconInput,
    MVDeconvolution,
)
from .inputs import WeightNormalizer, WeightType, transform_input  # noqa: F401,E402
from .separable import CUDASeparableConvolution, CUDASeparableConvolutionFunctions, OutOfBounds  # noqa: F401,E402
from .psf import ExtractPSF  # noqa: F401,E402
from .export import Save3dTIFF  # noqa: F401,E402
