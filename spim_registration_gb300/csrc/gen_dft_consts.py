"""Writes dft_consts.cuh: exp(-2 pi i m / R) for the composite register DFT sizes.

The values are the roots of unity computed here in double precision and rounded to float.
Run:  python spim_registration_gb300/csrc/gen_dft_consts.py
"""
import math
import os

SIZES = [6, 8, 9, 10, 12, 14, 15, 16, 18, 20]
out = ["// Generated by gen_dft_consts.py: W_R^m = exp(-2 pi i m / R) for composite R.",
       "#pragma once", "#include <cuda_runtime.h>", "", "namespace mvd {", ""]
for r in SIZES:
    vals = []
    for m in range(r):
        a = -2.0 * math.pi * m / r
        vals.append("{%.9ef, %.9ef}" % (math.cos(a), math.sin(a)))
    out.append(f"static __constant__ float2 c_w{r}[{r}] = {{" + ", ".join(vals) + "};")
out += ["", "template <int R>", "__device__ __forceinline__ float2 wconst(int m);"]
for r in SIZES:
    out.append(f"template <> __device__ __forceinline__ float2 wconst<{r}>(int m) {{ return c_w{r}[m]; }}")
out += ["", "}  // namespace mvd", ""]
path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dft_consts.cuh")
open(path, "w").write("\n".join(out))
print(path)
