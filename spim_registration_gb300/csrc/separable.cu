// Separable 3D convolution: the native interface the interest-point detection binds through
// JNA (spim/process/cuda/CUDASeparableConvolution.java:34-46), used for the Gaussians of the
// difference-of-Gaussian detector (spim/process/cuda/CUDASeparableConvolutionFunctions.java:148-210,
// spim/process/interestpointdetection/DifferenceOfGaussianCUDA.java:137-196).
//
// convolve_K(image, kx, ky, kz, w, h, d, cx, cy, cz, oob, value, dev) convolves the image in
// place along x, then y, then z (each axis only when its flag is set) with kernels of K taps
// (K in {7, 15, 31, 63, 127}; the caller centres shorter kernels in zeros).  Every pass
// extends its own input at the image border: 0 = zero, 1 = `value`, 2 = the border pixel.
// out[x] = sum_{j=-R..R} in[x + j] k[R - j] (R = K / 2), accumulated in float in order of j.
//
// GPU layout: one pass per axis, out of place between two device buffers.
//  * x pass: a CTA loads a row segment and its halo into shared memory (coalesced), each
//    thread computes PX consecutive outputs from a sliding register window.
//  * y / z pass: a CTA loads a 32-wide (x) slab of CH axis positions plus the halo into shared
//    memory (each warp reads 32 consecutive floats of one axis position), each thread computes
//    PA consecutive outputs along the axis for its x.
// Taps travel as kernel parameters (uniform reads from the constant bank).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mvdecon.h"
#include "engine.h"

using namespace mvd;

namespace mvd {
void set_last_error(const std::string& msg);
}

namespace {

constexpr int kMaxTaps = 127;

struct Taps {
  float k[kMaxTaps];  // flipped: t[m] = kernel[2R - m], so out[x] = sum_m in[x - R + m] t[m]
};

enum Oob { OOB_ZERO = 0, OOB_VALUE = 1, OOB_EXTEND = 2 };

__device__ __forceinline__ float fetch(const float* __restrict__ p, long long base, long long stride, int i, int n,
                                       int oob, float value) {
  if (i >= 0 && i < n) return __ldg(p + base + (long long)i * stride);
  if (oob == OOB_EXTEND) return __ldg(p + base + (long long)(i < 0 ? 0 : n - 1) * stride);
  return oob == OOB_VALUE ? value : 0.f;
}

// ---- x pass --------------------------------------------------------------------------------
constexpr int kPX = 4;       // outputs per thread
constexpr int kXThreads = 128;

template <int R>
__global__ void __launch_bounds__(kXThreads) sep_x_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                          int w, long long rows, Taps taps, int oob, float value) {
  constexpr int SEG = kXThreads * kPX;
  __shared__ float s[SEG + 2 * R + 1];
  const long long row = blockIdx.y + (long long)blockIdx.z * gridDim.y;
  if (row >= rows) return;
  const int x0 = blockIdx.x * SEG;
  const long long base = row * (long long)w;
  for (int i = threadIdx.x; i < SEG + 2 * R + 1; i += kXThreads) s[i] = fetch(in, base, 1, x0 - R + i, w, oob, value);
  __syncthreads();
  const int xl = threadIdx.x * kPX;
  if (x0 + xl >= w) return;
  float acc[kPX];
  float win[kPX];
#pragma unroll
  for (int o = 0; o < kPX; ++o) {
    acc[o] = 0.f;
    win[o] = s[xl + o];
  }
#pragma unroll 8
  for (int m = 0; m <= 2 * R; ++m) {
    const float t = taps.k[m];
#pragma unroll
    for (int o = 0; o < kPX; ++o) acc[o] = __fmaf_rn(win[o], t, acc[o]);
#pragma unroll
    for (int o = 0; o < kPX - 1; ++o) win[o] = win[o + 1];
    win[kPX - 1] = s[xl + kPX + m];
  }
#pragma unroll
  for (int o = 0; o < kPX; ++o)
    if (x0 + xl + o < w) out[base + x0 + xl + o] = acc[o];
}

// ---- y / z pass ----------------------------------------------------------------------------
constexpr int kAWarps = 8;
constexpr int kPA = 8;                 // outputs per thread along the axis
constexpr int kCH = kAWarps * kPA;     // axis outputs per CTA

// Element (x, a, o) at x + a * sa + o * so; the axis a has length n.
template <int R>
__global__ void __launch_bounds__(32 * kAWarps) sep_axis_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                                 int w, int n, long long sa, long long so, Taps taps,
                                                                 int oob, float value) {
  __shared__ float s[(kCH + 2 * R + 1) * 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int x = blockIdx.x * 32 + lane;
  const int a0 = blockIdx.y * kCH;
  const long long o = blockIdx.z;
  const bool xin = x < w;
  const long long base = (long long)(xin ? x : 0) + o * so;
  for (int r = warp; r < kCH + 2 * R + 1; r += kAWarps)
    s[r * 32 + lane] = xin ? fetch(in, base, sa, a0 - R + r, n, oob, value) : 0.f;
  __syncthreads();
  if (!xin) return;
  const int al = warp * kPA;
  if (a0 + al >= n) return;
  float acc[kPA];
  float win[kPA];
#pragma unroll
  for (int q = 0; q < kPA; ++q) {
    acc[q] = 0.f;
    win[q] = s[(al + q) * 32 + lane];
  }
#pragma unroll 8
  for (int m = 0; m <= 2 * R; ++m) {
    const float t = taps.k[m];
#pragma unroll
    for (int q = 0; q < kPA; ++q) acc[q] = __fmaf_rn(win[q], t, acc[q]);
#pragma unroll
    for (int q = 0; q < kPA - 1; ++q) win[q] = win[q + 1];
    win[kPA - 1] = s[(al + kPA + m) * 32 + lane];
  }
#pragma unroll
  for (int q = 0; q < kPA; ++q)
    if (a0 + al + q < n) out[base + (long long)(a0 + al + q) * sa] = acc[q];
}

// The sliding window loads one element past the last tap (win[P-1] after the last FMA), so
// the shared buffers carry one extra slot: x holds SEG + 2R + 1 elements (the last thread
// reads up to index SEG - PX + PX + 2R), the axis slab CH + 2R + 1 rows.

template <int R>
void launch_pass(int axis, const float* in, float* out, int w, int h, int d, const Taps& t, int oob, float value,
                 cudaStream_t s) {
  if (axis == 0) {
    const long long rows = (long long)h * d;
    const int gx = (w + kXThreads * kPX - 1) / (kXThreads * kPX);
    const long long gy = std::min<long long>(rows, 65535);
    const long long gz = (rows + gy - 1) / gy;
    sep_x_kernel<R><<<dim3(gx, (unsigned)gy, (unsigned)gz), kXThreads, 0, s>>>(in, out, w, rows, t, oob, value);
  } else {
    const int n = axis == 1 ? h : d;
    const long long sa = axis == 1 ? (long long)w : (long long)w * h;
    const long long so = axis == 1 ? (long long)w * h : (long long)w;
    const int outer = axis == 1 ? d : h;
    if (outer > 65535 || (n + kCH - 1) / kCH > 65535) throw std::invalid_argument("image too large for the y/z passes");
    sep_axis_kernel<R><<<dim3((w + 31) / 32, (n + kCH - 1) / kCH, outer), 32 * kAWarps, 0, s>>>(in, out, w, n, sa, so,
                                                                                             t, oob, value);
  }
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

void run_pass(int taps_len, int axis, const float* in, float* out, int w, int h, int d, const Taps& t, int oob,
              float value, cudaStream_t s) {
  switch (taps_len) {
    case 7: launch_pass<3>(axis, in, out, w, h, d, t, oob, value, s); break;
    case 15: launch_pass<7>(axis, in, out, w, h, d, t, oob, value, s); break;
    case 31: launch_pass<15>(axis, in, out, w, h, d, t, oob, value, s); break;
    case 63: launch_pass<31>(axis, in, out, w, h, d, t, oob, value, s); break;
    case 127: launch_pass<63>(axis, in, out, w, h, d, t, oob, value, s); break;
    default: throw std::invalid_argument("unsupported kernel size");
  }
}

Taps flip_taps(const float* k, int len) {
  Taps t{};
  for (int m = 0; m < len; ++m) t.k[m] = k[len - 1 - m];
  return t;
}

// A kernel of 2r + 1 taps centred in the smallest supported size (zeros around it).
int supported_size(int taps) {
  for (int s : {7, 15, 31, 63, 127})
    if (taps <= s) return s;
  return -1;
}

std::vector<float> centred(const float* k, int len, int size) {
  std::vector<float> out(size, 0.f);
  const int o = (size - len) / 2;
  for (int i = 0; i < len; ++i) out[o + i] = k[i];
  return out;
}

// The passes of one convolution over device buffers a (input) and b (scratch); returns the
// buffer that holds the result.
float* convolve_device(float* a, float* b, int w, int h, int d, const float* const k[3], const int len[3],
                       int oob, float value, cudaStream_t s) {
  float* src = a;
  float* dst = b;
  for (int axis = 0; axis < 3; ++axis) {
    if (!k[axis]) continue;
    const int size = supported_size(len[axis]);
    if (size < 0) throw std::invalid_argument("kernel longer than 127 taps");
    const std::vector<float> c = centred(k[axis], len[axis], size);
    run_pass(size, axis, src, dst, w, h, d, flip_taps(c.data(), size), oob, value, s);
    std::swap(src, dst);
  }
  return src;
}

struct SepCtx {
  std::mutex mu;
  cudaStream_t stream = nullptr;
  DevBuf a, b;
};

SepCtx& sep_ctx(int dev) {
  static std::mutex mu;
  static std::vector<std::unique_ptr<SepCtx>> ctxs;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)ctxs.size() <= dev) ctxs.resize(dev + 1);
  if (!ctxs[dev]) {
    ctxs[dev] = std::make_unique<SepCtx>();
    MVD_CHECK(cudaSetDevice(dev));
    MVD_CHECK(cudaStreamCreateWithFlags(&ctxs[dev]->stream, cudaStreamNonBlocking));
  }
  return *ctxs[dev];
}

int check_args(const float* image, int w, int h, int d, int oob) {
  if (!image) {
    set_last_error("image is NULL");
    return MVD_ERR_ARG;
  }
  if (w < 1 || h < 1 || d < 1) {
    set_last_error("image sizes must be positive");
    return MVD_ERR_ARG;
  }
  if (oob < 0 || oob > 2) {
    set_last_error("outofbounds must be 0 (zero), 1 (value) or 2 (extend border pixels)");
    return MVD_ERR_ARG;
  }
  return MVD_OK;
}

// Host image in, host image out (the JNA calls).
int convolve_host(float* image, const float* const k[3], const int len[3], int w, int h, int d, int oob, float value,
                  int dev) {
  try {
    set_last_error("");
    int st = check_args(image, w, h, d, oob);
    if (st != MVD_OK) return st;
    int count = 0;
    MVD_CHECK(cudaGetDeviceCount(&count));
    // the CPU request (devCUDA = -1) runs on GPU 0: this library has no CPU code path
    if (dev < 0) dev = 0;
    if (dev >= count) {
      set_last_error("invalid CUDA device id");
      return MVD_ERR_ARG;
    }
    SepCtx& c = sep_ctx(dev);
    std::lock_guard<std::mutex> lock(c.mu);
    MVD_CHECK(cudaSetDevice(dev));
    const size_t bytes = (size_t)w * h * d * sizeof(float);
    c.a.ensure(bytes);
    c.b.ensure(bytes);
    MVD_CHECK(cudaMemcpyAsync(c.a.p, image, bytes, cudaMemcpyHostToDevice, c.stream));
    float* res = convolve_device(c.a.as<float>(), c.b.as<float>(), w, h, d, k, len, oob, value, c.stream);
    MVD_CHECK(cudaMemcpyAsync(image, res, bytes, cudaMemcpyDeviceToHost, c.stream));
    MVD_CHECK(cudaStreamSynchronize(c.stream));
    return MVD_OK;
  } catch (const CudaError& e) {
    set_last_error(e.what());
    return MVD_ERR_CUDA;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return MVD_ERR_INTERNAL;
  }
}

int convolve_fixed(int K, float* image, const float* kx, const float* ky, const float* kz, int w, int h, int d, int cx,
                   int cy, int cz, int oob, float value, int dev) {
  const float* k[3] = {cx ? kx : nullptr, cy ? ky : nullptr, cz ? kz : nullptr};
  const int len[3] = {K, K, K};
  for (int a = 0; a < 3; ++a)
    if ((a == 0 ? cx : a == 1 ? cy : cz) && !k[a]) {
      set_last_error("a kernel of an axis to convolve is NULL");
      return 0;
    }
  const int st = convolve_host(image, k, len, w, h, d, oob, value, dev);
  if (st != MVD_OK) std::fprintf(stderr, "convolve_%d: %s\n", K, mvd_last_error());
  return st == MVD_OK;
}

}  // namespace

extern "C" {

int convolve_127(float* image, float* kernelX, float* kernelY, float* kernelZ, int imageW, int imageH, int imageD,
                 int convolveX, int convolveY, int convolveZ, int outofbounds, float outofboundsvalue, int devCUDA) {
  return convolve_fixed(127, image, kernelX, kernelY, kernelZ, imageW, imageH, imageD, convolveX, convolveY,
                        convolveZ, outofbounds, outofboundsvalue, devCUDA);
}
int convolve_63(float* image, float* kernelX, float* kernelY, float* kernelZ, int imageW, int imageH, int imageD,
                int convolveX, int convolveY, int convolveZ, int outofbounds, float outofboundsvalue, int devCUDA) {
  return convolve_fixed(63, image, kernelX, kernelY, kernelZ, imageW, imageH, imageD, convolveX, convolveY,
                        convolveZ, outofbounds, outofboundsvalue, devCUDA);
}
int convolve_31(float* image, float* kernelX, float* kernelY, float* kernelZ, int imageW, int imageH, int imageD,
                int convolveX, int convolveY, int convolveZ, int outofbounds, float outofboundsvalue, int devCUDA) {
  return convolve_fixed(31, image, kernelX, kernelY, kernelZ, imageW, imageH, imageD, convolveX, convolveY,
                        convolveZ, outofbounds, outofboundsvalue, devCUDA);
}
int convolve_15(float* image, float* kernelX, float* kernelY, float* kernelZ, int imageW, int imageH, int imageD,
                int convolveX, int convolveY, int convolveZ, int outofbounds, float outofboundsvalue, int devCUDA) {
  return convolve_fixed(15, image, kernelX, kernelY, kernelZ, imageW, imageH, imageD, convolveX, convolveY,
                        convolveZ, outofbounds, outofboundsvalue, devCUDA);
}
int convolve_7(float* image, float* kernelX, float* kernelY, float* kernelZ, int imageW, int imageH, int imageD,
               int convolveX, int convolveY, int convolveZ, int outofbounds, float outofboundsvalue, int devCUDA) {
  return convolve_fixed(7, image, kernelX, kernelY, kernelZ, imageW, imageH, imageD, convolveX, convolveY,
                        convolveZ, outofbounds, outofboundsvalue, devCUDA);
}

void convolutionCPU(float* image, float* kernelX, float* kernelY, float* kernelZ, int kernelRX, int kernelRY,
                    int kernelRZ, int imageW, int imageH, int imageD, int outofbounds, float outofboundsvalue) {
  if (kernelRX < 0 || kernelRY < 0 || kernelRZ < 0 || kernelRX > 63 || kernelRY > 63 || kernelRZ > 63 || !kernelX ||
      !kernelY || !kernelZ) {
    set_last_error("kernel radii must be in [0, 63] with all three kernels given");
    std::fprintf(stderr, "convolutionCPU: %s\n", mvd_last_error());
    return;
  }
  const float* k[3] = {kernelX, kernelY, kernelZ};
  const int len[3] = {2 * kernelRX + 1, 2 * kernelRY + 1, 2 * kernelRZ + 1};
  if (convolve_host(image, k, len, imageW, imageH, imageD, outofbounds, outofboundsvalue, -1) != MVD_OK)
    std::fprintf(stderr, "convolutionCPU: %s\n", mvd_last_error());
}

int mvd_separable_convolve_device(float* image, float* scratch, const float* const* kernels, const int* taps,
                                  const int* dims_xyz, int outofbounds, float outofboundsvalue, int devCUDA,
                                  void* stream, float** result) {
  try {
    set_last_error("");
    if (!dims_xyz || !kernels || !taps || !scratch || !result) {
      set_last_error("NULL argument");
      return MVD_ERR_ARG;
    }
    int st = check_args(image, dims_xyz[0], dims_xyz[1], dims_xyz[2], outofbounds);
    if (st != MVD_OK) return st;
    const float* k[3];
    int len[3];
    for (int a = 0; a < 3; ++a) {
      k[a] = kernels[a];
      len[a] = taps[a];
      if (k[a] && (len[a] < 1 || !(len[a] & 1) || len[a] > kMaxTaps)) {
        set_last_error("kernel lengths must be odd and at most 127");
        return MVD_ERR_ARG;
      }
    }
    MVD_CHECK(cudaSetDevice(devCUDA));
    *result = convolve_device(image, scratch, dims_xyz[0], dims_xyz[1], dims_xyz[2], k, len, outofbounds,
                              outofboundsvalue, static_cast<cudaStream_t>(stream));
    return MVD_OK;
  } catch (const CudaError& e) {
    set_last_error(e.what());
    return MVD_ERR_CUDA;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return MVD_ERR_INTERNAL;
  }
}

}  // extern "C"
