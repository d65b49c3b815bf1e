// PSF pipeline on the GPU: extraction of the point spread function from bead neighbourhoods
// and its transformation into the fused frame.
//   ExtractPSF.extractPSFLocal  spim/process/fusion/deconvolution/ExtractPSF.java:374-415
//   ExtractPSF.normalize        :298-316
//   ExtractPSF.transformPSF     :325-372
//   ExtractPSF.transform        :417-464
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <string>

#include "../../include/mvdecon.h"
#include "engine.h"

using namespace mvd;

namespace mvd {
void set_last_error(const std::string& msg);
}

namespace {

__device__ __forceinline__ int periodic(int i, int n) {
  int m = i % n;
  return m < 0 ? m + n : m;
}

// Trilinear interpolation at (tx, ty, tz) of the volume extended periodically (PERIODIC) or
// with zeros; the corner weights come from the fractional parts, the sum is in float.
template <bool PERIODIC>
__device__ __forceinline__ float trilinear(const float* __restrict__ v, int sx, int sy, int sz, double tx, double ty,
                                           double tz) {
  const double fx = floor(tx), fy = floor(ty), fz = floor(tz);
  const int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
  const float ax = (float)(tx - fx), ay = (float)(ty - fy), az = (float)(tz - fz);
  float acc = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int bx = c & 1, by = (c >> 1) & 1, bz = (c >> 2) & 1;
    int x = x0 + bx, y = y0 + by, z = z0 + bz;
    float val;
    if (PERIODIC) {
      x = periodic(x, sx);
      y = periodic(y, sy);
      z = periodic(z, sz);
      val = __ldg(v + ((long long)z * sy + y) * sx + x);
    } else {
      val = (x >= 0 && y >= 0 && z >= 0 && x < sx && y < sy && z < sz) ? __ldg(v + ((long long)z * sy + y) * sx + x)
                                                                       : 0.f;
    }
    const float w = (bx ? ax : 1.f - ax) * (by ? ay : 1.f - ay) * (bz ? az : 1.f - az);
    acc = __fmaf_rn(w, val, acc);
  }
  return acc;
}

// One thread per PSF voxel; the bead locations are summed in their given order (as the
// reference adds them voxel by voxel, location after location).
__global__ void extract_psf_kernel(const float* __restrict__ img, int sx, int sy, int sz,
                                   const double* __restrict__ loc, int n, int px, int py, int pz,
                                   float* __restrict__ psf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= px * py * pz) return;
  const int x = i % px, y = (i / px) % py, z = i / (px * py);
  const double ox = x - px / 2, oy = y - py / 2, oz = z - pz / 2;
  float acc = 0.f;
  for (int l = 0; l < n; ++l)
    acc += trilinear<true>(img, sx, sy, sz, ox + loc[3 * l], oy + loc[3 * l + 1], oz + loc[3 * l + 2]);
  psf[i] = acc;
}

// (v - min) / (max - min) in double, min and max over the whole PSF (one CTA: PSFs are small)
__global__ void normalize_min_max_kernel(float* __restrict__ p, int n) {
  __shared__ double smin[32], smax[32];
  double lo = DBL_MAX, hi = -DBL_MAX;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = p[i];
    lo = fmin(lo, v);
    hi = fmax(hi, v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    smin[warp] = lo;
    smax[warp] = hi;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    lo = lane < nw ? smin[lane] : DBL_MAX;
    hi = lane < nw ? smax[lane] : -DBL_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (lane == 0) {
      smin[0] = lo;
      smax[0] = hi;
    }
  }
  __syncthreads();
  lo = smin[0];
  hi = smax[0];
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = (float)(((double)p[i] - lo) / (hi - lo));
}

struct Affine64 {
  double m[12];
};

// out[p] = psf(model^-1 (p + offset)), trilinear over the PSF extended with zeros
__global__ void transform_psf_kernel(const float* __restrict__ psf, int sx, int sy, int sz, Affine64 inv,
                                     double offx, double offy, double offz, int nx, int ny, int nz,
                                     float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nx * ny * nz) return;
  const int x = i % nx, y = (i / nx) % ny, z = i / (nx * ny);
  const double p0 = x + offx, p1 = y + offy, p2 = z + offz;
  const double t0 = inv.m[0] * p0 + inv.m[1] * p1 + inv.m[2] * p2 + inv.m[3];
  const double t1 = inv.m[4] * p0 + inv.m[5] * p1 + inv.m[6] * p2 + inv.m[7];
  const double t2 = inv.m[8] * p0 + inv.m[9] * p1 + inv.m[10] * p2 + inv.m[11];
  out[i] = trilinear<false>(psf, sx, sy, sz, t0, t1, t2);
}

bool invert(const double* a, Affine64& out) {
  const double r00 = a[0], r01 = a[1], r02 = a[2], r10 = a[4], r11 = a[5], r12 = a[6], r20 = a[8], r21 = a[9],
               r22 = a[10];
  const double det = r00 * (r11 * r22 - r12 * r21) - r01 * (r10 * r22 - r12 * r20) + r02 * (r10 * r21 - r11 * r20);
  if (!(std::fabs(det) > 0.0)) return false;
  const double inv[9] = {(r11 * r22 - r12 * r21) / det, (r02 * r21 - r01 * r22) / det, (r01 * r12 - r02 * r11) / det,
                         (r12 * r20 - r10 * r22) / det, (r00 * r22 - r02 * r20) / det, (r02 * r10 - r00 * r12) / det,
                         (r10 * r21 - r11 * r20) / det, (r01 * r20 - r00 * r21) / det, (r00 * r11 - r01 * r10) / det};
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) out.m[4 * r + c] = inv[3 * r + c];
    out.m[4 * r + 3] = -(inv[3 * r] * a[3] + inv[3 * r + 1] * a[7] + inv[3 * r + 2] * a[11]);
  }
  return true;
}

int blocks_for(long long n) { return (int)((n + 255) / 256); }

}  // namespace

extern "C" int mvd_transformed_psf_size(const int* psf_dims, const double* model, int* out_dims, double* offset) {
  set_last_error("");
  if (!psf_dims || !model || !out_dims || !offset) {
    set_last_error("NULL argument");
    return MVD_ERR_ARG;
  }
  for (int d = 0; d < 3; ++d)
    if (psf_dims[d] < 1) {
      set_last_error("PSF sizes must be positive");
      return MVD_ERR_ARG;
    }
  // estimateBounds of the interval [0, dim - 1]: the bounding box of its 8 transformed corners
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int c = 0; c < 8; ++c) {
    const double p[3] = {(c & 1) ? psf_dims[0] - 1.0 : 0.0, (c & 2) ? psf_dims[1] - 1.0 : 0.0,
                         (c & 4) ? psf_dims[2] - 1.0 : 0.0};
    for (int d = 0; d < 3; ++d) {
      const double t = model[4 * d] * p[0] + model[4 * d + 1] * p[1] + model[4 * d + 2] * p[2] + model[4 * d + 3];
      lo[d] = std::fmin(lo[d], t);
      hi[d] = std::fmax(hi[d], t);
    }
  }
  // the PSF's centre voxel (dim / 2, integer) maps to the centre of the odd-sized result
  const double ctr[3] = {(double)(psf_dims[0] / 2), (double)(psf_dims[1] / 2), (double)(psf_dims[2] / 2)};
  for (int d = 0; d < 3; ++d) {
    long long ns = (long long)(hi[d] - lo[d]) + 1;
    if (ns % 2 == 0) ++ns;
    if (ns > (1 << 20)) {
      set_last_error("transformed PSF too large");
      return MVD_ERR_ARG;
    }
    out_dims[d] = (int)ns;
    const double tc = model[4 * d] * ctr[0] + model[4 * d + 1] * ctr[1] + model[4 * d + 2] * ctr[2] + model[4 * d + 3];
    offset[d] = tc - (double)(ns / 2);
  }
  return MVD_OK;
}

extern "C" int mvd_extract_psf(const float* img, const int* dims, const double* locations, int num_locations,
                               const int* psf_dims, float* psf, int normalize, int devCUDA, void* stream) {
  try {
    set_last_error("");
    if (!img || !dims || !psf_dims || !psf || (num_locations > 0 && !locations) || num_locations < 0) {
      set_last_error("NULL argument or negative location count");
      return MVD_ERR_ARG;
    }
    for (int d = 0; d < 3; ++d)
      if (dims[d] < 1 || psf_dims[d] < 1) {
        set_last_error("sizes must be positive");
        return MVD_ERR_ARG;
      }
    const long long np = (long long)psf_dims[0] * psf_dims[1] * psf_dims[2];
    if (np > (1LL << 30)) {
      set_last_error("PSF too large");
      return MVD_ERR_ARG;
    }
    MVD_CHECK(cudaSetDevice(devCUDA));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void* d_loc = nullptr;
    const size_t lb = (size_t)(num_locations > 0 ? num_locations : 1) * 3 * sizeof(double);
    MVD_CHECK(cudaMallocAsync(&d_loc, lb, s));
    if (num_locations > 0)
      MVD_CHECK(cudaMemcpyAsync(d_loc, locations, (size_t)num_locations * 3 * sizeof(double), cudaMemcpyHostToDevice,
                                s));
    extract_psf_kernel<<<blocks_for(np), 256, 0, s>>>(img, dims[0], dims[1], dims[2], static_cast<double*>(d_loc),
                                                      num_locations, psf_dims[0], psf_dims[1], psf_dims[2], psf);
    MVD_CHECK(cudaGetLastError());
    count_launch();
    if (normalize) {
      normalize_min_max_kernel<<<1, 1024, 0, s>>>(psf, (int)np);
      MVD_CHECK(cudaGetLastError());
      count_launch();
    }
    MVD_CHECK(cudaFreeAsync(d_loc, s));
    return MVD_OK;
  } catch (const CudaError& e) {
    set_last_error(e.what());
    return MVD_ERR_CUDA;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return MVD_ERR_INTERNAL;
  }
}

extern "C" int mvd_transform_psf(const float* psf, const int* psf_dims, const double* model, const int* out_dims,
                                 const double* offset, float* out, int devCUDA, void* stream) {
  try {
    set_last_error("");
    if (!psf || !psf_dims || !model || !out_dims || !offset || !out) {
      set_last_error("NULL argument");
      return MVD_ERR_ARG;
    }
    for (int d = 0; d < 3; ++d)
      if (psf_dims[d] < 1 || out_dims[d] < 1) {
        set_last_error("sizes must be positive");
        return MVD_ERR_ARG;
      }
    const long long no = (long long)out_dims[0] * out_dims[1] * out_dims[2];
    if (no > (1LL << 30)) {
      set_last_error("output too large");
      return MVD_ERR_ARG;
    }
    Affine64 inv;
    if (!invert(model, inv)) {
      set_last_error("the affine transform is singular");
      return MVD_ERR_ARG;
    }
    MVD_CHECK(cudaSetDevice(devCUDA));
    transform_psf_kernel<<<blocks_for(no), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        psf, psf_dims[0], psf_dims[1], psf_dims[2], inv, offset[0], offset[1], offset[2], out_dims[0], out_dims[1],
        out_dims[2], out);
    MVD_CHECK(cudaGetLastError());
    count_launch();
    return MVD_OK;
  } catch (const CudaError& e) {
    set_last_error(e.what());
    return MVD_ERR_CUDA;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return MVD_ERR_INTERNAL;
  }
}
