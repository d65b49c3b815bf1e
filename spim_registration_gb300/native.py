"""ctypes binding of ``libFourierConvolutionCUDA.so`` -- the way JNA binds it from Java.

JNA maps each Java interface method to the C symbol of the same name and marshals ``float[]``
as a pointer to a temporary native copy; here numpy float32 C-contiguous arrays play that
role.  There is no CPU fallback: if the library is missing or cannot be loaded, every call
raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import _build

_lib = None
_lock = threading.Lock()

MVD_OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "invalid state",
          5: "internal error"}


class MvdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


_F = ctypes.POINTER(ctypes.c_float)
_I = ctypes.POINTER(ctypes.c_int)
_D = ctypes.POINTER(ctypes.c_double)
_LL = ctypes.POINTER(ctypes.c_longlong)
_H = ctypes.c_void_p

# name -> (restype, argtypes); every symbol declared in include/mvdecon.h
SIGNATURES = {
    "getCUDAcomputeCapabilityMinorVersion": (ctypes.c_int, [ctypes.c_int]),
    "getCUDAcomputeCapabilityMajorVersion": (ctypes.c_int, [ctypes.c_int]),
    "getNumDevicesCUDA": (ctypes.c_int, []),
    "getNameDeviceCUDA": (None, [ctypes.c_int, ctypes.c_char_p]),
    "getMemDeviceCUDA": (ctypes.c_longlong, [ctypes.c_int]),
    "getFreeMemDeviceCUDA": (ctypes.c_longlong, [ctypes.c_int]),
    "convolution3DfftCUDA": (_F, [_F, _I, _F, _I, ctypes.c_int]),
    "convolution3DfftCUDAInPlace": (None, [_F, _I, _F, _I, ctypes.c_int]),
    "mvd_last_error": (ctypes.c_char_p, []),
    "mvd_version": (ctypes.c_char_p, []),
    "mvd_convolve3d_inplace": (ctypes.c_int, [_F, _I, _F, _I, ctypes.c_int]),
    "mvd_convolve3d_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, _I, ctypes.c_void_p, _I,
                                             ctypes.c_int, ctypes.c_float, ctypes.c_int, ctypes.c_void_p]),
    "mvd_convolve3d_device_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, _I, ctypes.c_void_p, _I,
                                                     ctypes.c_int, ctypes.c_float, ctypes.c_int, ctypes.c_void_p]),
    "mvd_create": (ctypes.c_int, [ctypes.POINTER(_H), ctypes.c_int, _I, ctypes.c_int, ctypes.POINTER(_F),
                                  ctypes.POINTER(_F), ctypes.POINTER(_F), _I, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_int, _I]),
    "mvd_destroy": (ctypes.c_int, [_H]),
    "mvd_run_view": (ctypes.c_int, [_H, ctypes.c_int]),
    "mvd_run_iteration": (ctypes.c_int, [_H]),
    "mvd_run": (ctypes.c_int, [_H, ctypes.c_int]),
    "mvd_synchronize": (ctypes.c_int, [_H]),
    "mvd_get_psi": (ctypes.c_int, [_H, _F, ctypes.c_int]),
    "mvd_set_psi": (ctypes.c_int, [_H, _F]),
    "mvd_get_initial_average": (ctypes.c_int, [_H, _D]),
    "mvd_get_kernel": (ctypes.c_int, [_H, ctypes.c_int, ctypes.c_int, _F]),
    "mvd_get_stats": (ctypes.c_int, [_H, ctypes.c_int, ctypes.c_int, _D, _D]),
    "mvd_get_iteration": (ctypes.c_int, [_H, _I]),
    "mvd_get_plan": (ctypes.c_int, [_H, ctypes.c_int, _I, _I, _I, _LL]),
    "mvd_get_plan_variant": (ctypes.c_int, [_H, ctypes.c_int, _I, _I]),
    "mvd_get_stream": (ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_void_p)]),
    "mvd_get_launch_count": (ctypes.c_int, [_H, _LL]),
    "mvd_profile_iteration": (ctypes.c_int, [_H, _D, _I]),
    "mvd_forward": (ctypes.c_int, [_H, _D]),
    "mvd_backward": (ctypes.c_int, [_H, _F, ctypes.POINTER(_F)]),
    "mvd_set_kernel": (ctypes.c_int, [_H, ctypes.c_int, ctypes.c_int, _F]),
    "mvd_transform_view": (ctypes.c_int, [ctypes.c_void_p, _I, _D, _I, _I, ctypes.c_void_p, ctypes.c_void_p, _F, _F,
                                          ctypes.c_int, ctypes.c_void_p]),
    "mvd_normalize_weights": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_longlong,
                                             ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "mvd_weight_overlap": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_longlong, ctypes.c_int,
                                          _I, ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_void_p]),
    **{f"convolve_{k}": (ctypes.c_int, [_F, _F, _F, _F, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int])
       for k in (127, 63, 31, 15, 7)},
    "convolutionCPU": (None, [_F, _F, _F, _F, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, ctypes.c_int, ctypes.c_float]),
    "mvd_extract_psf": (ctypes.c_int, [ctypes.c_void_p, _I, _D, ctypes.c_int, _I, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_void_p]),
    "mvd_transformed_psf_size": (ctypes.c_int, [_I, _D, _I, _D]),
    "mvd_transform_psf": (ctypes.c_int, [ctypes.c_void_p, _I, _D, _I, _D, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_void_p]),
    "mvd_separable_convolve_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(_F), _I, _I,
                                                     ctypes.c_int, ctypes.c_float, ctypes.c_int, ctypes.c_void_p,
                                                     ctypes.POINTER(ctypes.c_void_p)]),
}


def header_symbols() -> list[str]:
    """Function names declared in include/mvdecon.h (the C ABI contract)."""
    import re

    path = os.path.join(os.path.dirname(_build.PKG), "include", "mvdecon.h")
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"^[ \t]*#.*$", "", text, flags=re.M)  # preprocessor lines (function-like macros)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return [n for n in names if n not in ("if", "while", "sizeof")]


def load(path: str | None = None, build_if_missing: bool = False):
    """Load the library (once).  Raises if it is absent: there is no fallback."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or _build.library_path()
        if not os.path.exists(p):
            if build_if_missing:
                _build.build()
            else:
                raise RuntimeError(f"{p} is missing: build it with spim_registration_gb300._build.build()")
        lib = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int):
    if status != MVD_OK:
        msg = load().mvd_last_error().decode(errors="replace")
        raise MvdError(status, msg)


def fptr(a: np.ndarray):
    if a.dtype != np.float32 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float32 array")
    return a.ctypes.data_as(_F)


def iarr(values):
    return (ctypes.c_int * len(values))(*values)
