"""Build step of the sm_103a library (nvcc, in-tree, no cmake).

Compiles ``csrc/*.cu`` in parallel for ``sm_103a`` and links ``lib/libFourierConvolutionCUDA.so``
(CUDA runtime linked statically, so the library needs only the driver), plus the aliases
``libConvolution3D_fftCUDAlib.so`` under which the legacy Fiji plugin loads the same ABI and
``libSeparableConvolutionCUDALib.so`` (the interest-point detection loads the separable
convolution from a file whose name contains "separable").
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
LIBNAME = "libFourierConvolutionCUDA.so"
ALIASES = ["libConvolution3D_fftCUDAlib.so", "libSeparableConvolutionCUDALib.so"]
SOURCES = ["engine.cu", "passes_fwd.cu", "passes_inv.cu", "passes_z.cu", "adjoint.cu", "inputs.cu", "psf.cu", "separable.cu",
           "capi.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-Xptxas", "-O3"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def library_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(PKG), "include", "mvdecon.h"))
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(LIBDIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc(), *ARCH, *FLAGS, "-c", s, "-o", o]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for out in ex.map(run, jobs):
            if verbose and out:
                sys.stderr.write(out)
    lib = library_path()
    if force or jobs or _stale(lib, objs):
        run([nvcc(), *ARCH, "-shared", "-o", lib, *objs])
    for name in ALIASES:
        alias = os.path.join(LIBDIR, name)
        if os.path.lexists(alias):
            os.remove(alias)
        os.symlink(LIBNAME, alias)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
