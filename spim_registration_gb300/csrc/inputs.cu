// Input preparation of the deconvolution on the GPU: every view resampled into the fused box
// with its blending weight, and the VIRTUAL weight normalisation with the OSEM factor.
//   TransformInput.loop         spim/process/fusion/deconvolution/TransformInput.java:90-116
//   TransformWeights.call       spim/process/fusion/deconvolution/TransformWeights.java
//   BlendingRealRandomAccess    spim/process/fusion/weights/BlendingRealRandomAccess.java:44-121
//   WeightNormalizer (VIRTUAL)  spim/process/fusion/deconvolution/WeightNormalizer.java:73-253,
//                               spim/process/fusion/weights/NormalizingRandomAccess.java:57-66
//   OSEM factor                 ProcessForDeconvolution.java:372-405
#include <climits>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/mvdecon.h"
#include "engine.h"

using namespace mvd;

namespace mvd {
void set_last_error(const std::string& msg);
}

namespace {

struct Affine {  // world -> view (the inverse of the view's registration), row-packed 3x4
  float m[12];
};

// BlendingRealRandomAccess's 1001-entry lookup table of (cos((1 - d) pi) + 1) / 2, in global
// memory read through L1 (each thread looks up its own entry, which the constant cache would
// serialise across a warp): as doubles, and as float pairs hi + lo with hi = (float)L and
// lo = (float)(L - hi), within 2^-48 relative of the double L
__device__ double g_blend_lut[1001];
__device__ float2 g_blend_pair[1001];

__device__ __forceinline__ int mirror_single_i(int i, int n) {
  if (i >= 0 && i < n) return i;
  if (n == 1) return 0;
  const int period = 2 * n - 2;
  int m = i % period;
  if (m < 0) m += period;
  return m < n ? m : period - m;
}

// NLinearInterpolator over Views.extendMirrorSingle(img) at the real position t; Index is the
// voxel index type (32-bit when the view holds fewer than 2^31 voxels)
template <class Index>
__device__ __forceinline__ float trilinear_mirror(const float* __restrict__ img, int sx, int sy, int sz, float tx,
                                                  float ty, float tz) {
  const float fx0 = floorf(tx), fy0 = floorf(ty), fz0 = floorf(tz);
  const int x0 = (int)fx0, y0 = (int)fy0, z0 = (int)fz0;
  const float ax = tx - fx0, ay = ty - fy0, az = tz - fz0;
  const int xs[2] = {mirror_single_i(x0, sx), mirror_single_i(x0 + 1, sx)};
  const int ys[2] = {mirror_single_i(y0, sy), mirror_single_i(y0 + 1, sy)};
  const int zs[2] = {mirror_single_i(z0, sz), mirror_single_i(z0 + 1, sz)};
  float acc = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int bx = c & 1, by = (c >> 1) & 1, bz = (c >> 2) & 1;
    const float w = (bx ? ax : 1.f - ax) * (by ? ay : 1.f - ay) * (bz ? az : 1.f - az);
    acc += w * __ldg(img + ((Index)zs[bz] * sy + ys[by]) * sx + xs[bx]);
  }
  return acc;
}

// The reference normalises in double (and multiplies blending weights by a double table);
// GB300's FP64 pipe is a small fraction of its FP32 one.  The sum over the views is
// reproduced exactly in 64-bit integers (exact_view_sum below); the per-view quotients and
// OSEM products, and the blending products, are carried as unevaluated float pairs (hi + lo,
// within ~2^-44 relative of the exact value) built from error-free transformations, rounded
// once at the end.  Each rounding is certified: when the pair lies within 2^-14 of a half ulp
// from a rounding boundary (or the result is tiny or an inexact power of two), only the
// reference's double rounding decides it.  The normalisation leaves such voxels unwritten and
// appends them to a list (warp-aggregated atomics), which a second kernel finishes with the
// reference's double arithmetic, so no warp diverges into the double path.  They are rare for
// a generic OSEM factor (~1e-4) but common for decimal ones: w * 1.7 is an exact tie in
// rational arithmetic for ~5% of floats w, and the double 1.7 sits just beside it.

struct FF {  // hi + lo
  float hi, lo;
};

// y = the float nearest hi + lo; false when that rounding is not certain.  The pair must come
// from error-free steps on operands whose products did not underflow (nonzero operands of at
// least 2^-96, see tiny()); a zero pair is then an exact zero, and lo == 0 an exact hi.
__device__ __forceinline__ bool round_pair(FF x, float& y) {
  y = __fadd_rn(x.hi, x.lo);
  if (x.hi == 0.f && x.lo == 0.f) return true;
  const unsigned b = __float_as_uint(y);
  const unsigned ex = b & 0x7f800000u;
  if (ex <= (24u << 23) || ex == 0x7f800000u) return false;  // below 2^-102, infinite or NaN
  if (x.lo == 0.f) return true;
  if ((b & 0x007fffffu) == 0u) return false;  // a power of two: the half ulp below is smaller
  const float half_ulp = __uint_as_float(ex - (24u << 23));
  const float d = __fadd_rn(__fsub_rn(x.hi, y), x.lo);  // (hi + lo) - y; hi - y is exact
  return fabsf(d) < __fmul_rn(half_ulp, 0.99993896484375f);
}

// nonzero and below 2^-96: too small for the error-free steps (their error terms could
// underflow)
__device__ __forceinline__ bool tiny(float x) { return x != 0.f && (__float_as_uint(x) & 0x7f800000u) < (31u << 23); }

// w / (d.hi + d.lo) as a pair: q = fl(w / d.hi) is correctly rounded, so w - q d.hi is exact
// (an FMA); the remainder over d gives the low part.
__device__ __forceinline__ FF ff_quotient(float w, FF d) {
  const float q = __fdiv_rn(w, d.hi);
  const float r = __fsub_rn(__fmaf_rn(-q, d.hi, w), __fmul_rn(q, d.lo));
  return {q, __fmul_rn(r, __frcp_rn(d.hi))};
}

// (a.hi + a.lo) * (b.hi + b.lo) as a pair
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.hi, -p);
  return {p, __fadd_rn(e, __fadd_rn(__fmul_rn(a.hi, b.lo), __fmul_rn(a.lo, b.hi)))};
}

// BlendingRealRandomAccess.computeWeight (:91-121) on the view interval [0, size)
__device__ __forceinline__ float blend_weight(float lx, float ly, float lz, int sx, int sy, int sz, float3 border,
                                              float3 range) {
  const float loc[3] = {lx, ly, lz};
  const float dm1[3] = {(float)(sx - 1), (float)(sy - 1), (float)(sz - 1)};
  const float b[3] = {border.x, border.y, border.z};
  const float r[3] = {range.x, range.y, range.z};
  float w = 1.f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float l = loc[d];
    const float dist = fmaxf(0.f, fminf(l - b[d], dm1[d] - l - b[d]));
    if (dist == 0.f) return 0.f;
    // relDist = dist / blending, multiplied in only when below 1: dist >= blending makes the
    // quotient at least 1, so the division is needed only below the blending distance
    if (!(dist >= r[d])) {
      const float rel = dist / r[d];
      if (!(rel < 1.f)) continue;
      // indexFor(d) = Math.round(d * 1000.0): the double product of a float and 1000 is exact,
      // so the index is the exact round-half-up of rel * 1000, found in float by two FMA sign
      // tests around a first guess (each FMA rounds once, which keeps the sign)
      int idx = __float2int_rd(__fmaf_rn(rel, 1000.f, 0.5f));
      if (__fmaf_rn(rel, 1000.f, 0.5f - (float)idx) < 0.f)
        --idx;
      else if (__fmaf_rn(rel, 1000.f, -0.5f - (float)idx) >= 0.f)
        ++idx;
      idx = min(max(idx, 0), 1000);
      // minDistance *= lookUp[idx]: the float nearest the double-rounded double product,
      // certified from the float pair (the double rounding cannot move a product that lies
      // farther than 2^-14 half ulps from a float rounding boundary), else in double
      const float2 L = __ldg(g_blend_pair + idx);
      float y;
      if (round_pair(ff_mul(FF{w, 0.f}, FF{L.x, L.y}), y))
        w = y;
      else
        w = (float)((double)w * __ldg(g_blend_lut + idx));
    }
  }
  return w;
}

// Output voxel (x, y, z): the resampled view (0 outside it) and its blending weight.
template <class Index>
__device__ __forceinline__ void transform_voxel(const float* __restrict__ view, int sx, int sy, int sz,
                                                const Affine& inv, float s0, float s1, float s2, bool want_img,
                                                bool want_blend, float3 border, float3 range, float& v, float& wgt) {
  const float t0 = inv.m[0] * s0 + inv.m[1] * s1 + inv.m[2] * s2 + inv.m[3];
  const float t1 = inv.m[4] * s0 + inv.m[5] * s1 + inv.m[6] * s2 + inv.m[7];
  const float t2 = inv.m[8] * s0 + inv.m[9] * s1 + inv.m[10] * s2 + inv.m[11];
  v = 0.f;  // no image data (MVDeconvolution.computeQuotient reads 0 as "no data")
  if (want_img && t0 >= 0.f && t1 >= 0.f && t2 >= 0.f && t0 < (float)sx && t1 < (float)sy && t2 < (float)sz)
    v = fmaxf(1e-4f, trilinear_mirror<Index>(view, sx, sy, sz, t0, t1, t2));
  // the blending weight is defined everywhere (the border can be negative)
  wgt = want_blend ? blend_weight(t0, t1, t2, sx, sy, sz, border, range) : 0.f;
}

// One thread per output voxel; a block covers a 32 x 8 patch of one z plane, so a warp runs
// along output x.  For views whose x axis lies closer to output x than to output z.
template <class Index>
__global__ void __launch_bounds__(256) transform_view_kernel(const float* __restrict__ view, int sx, int sy, int sz,
                                                             Affine inv, int ox, int oy, int oz, int nx, int ny,
                                                             float* __restrict__ out_img,
                                                             float* __restrict__ out_blend, float3 border,
                                                             float3 range) {
  const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z;
  if (x >= nx || y >= ny) return;
  const long long i = ((long long)z * ny + y) * nx + x;
  float v, wgt;
  transform_voxel<Index>(view, sx, sy, sz, inv, (float)(x + ox), (float)(y + oy), (float)(z + oz), out_img != nullptr,
                         out_blend != nullptr, border, range, v, wgt);
  if (out_img) out_img[i] = v;
  if (out_blend) out_blend[i] = wgt;
}

// The same for views whose x axis lies closer to output z (a rotation near 90 degrees about
// y): a block covers 32 z x 32 x of one y row and a warp runs along output z, so its lanes
// read neighbouring voxels of one view row instead of 32 view planes.  The results are staged
// in shared memory (rows padded to 33: conflict-free both ways) and stored along x.
template <class Index>
__global__ void __launch_bounds__(256) transform_view_zfast_kernel(
    const float* __restrict__ view, int sx, int sy, int sz, Affine inv, int ox, int oy, int oz, int nx, int ny,
    int nz, float* __restrict__ out_img, float* __restrict__ out_blend, float3 border, float3 range) {
  __shared__ float s_img[32][33], s_w[32][33];  // [z][x] within the tile
  const int lane = threadIdx.x, warp = threadIdx.y;
  const int x0 = blockIdx.x * 32, y = blockIdx.y, z0 = blockIdx.z * 32;
  const int z = z0 + lane;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int xl = warp + 8 * k, x = x0 + xl;
    if (x < nx && z < nz) {
      float v, wgt;
      transform_voxel<Index>(view, sx, sy, sz, inv, (float)(x + ox), (float)(y + oy), (float)(z + oz),
                             out_img != nullptr, out_blend != nullptr, border, range, v, wgt);
      s_img[lane][xl] = v;
      s_w[lane][xl] = wgt;
    }
  }
  __syncthreads();
  const int x = x0 + lane;
  if (x >= nx) return;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int zl = warp + 8 * j, zz = z0 + zl;
    if (zz < nz) {
      const long long i = ((long long)zz * ny + y) * nx + x;
      if (out_img) out_img[i] = s_img[zl][lane];
      if (out_blend) out_blend[i] = s_w[zl][lane];
    }
  }
}

struct WeightPtrs {
  float* p[16];
};

// Math.min(1, x) of the reference: NaN stays NaN (fminf would return 1)
__device__ __forceinline__ float java_min1(float x) { return x != x ? x : fminf(1.f, x); }

// One voxel with the reference's own double arithmetic; the weights are read again from
// memory, which the certified pass has not written for this voxel.
__device__ __forceinline__ void normalize_voxel_double(const WeightPtrs& w, int nv, long long i, double osem,
                                                       int mode) {
  double sum = 0.0;
#pragma unroll
  for (int v = 0; v < 16; ++v)
    if (v < nv) sum += (double)w.p[v][i];
  const float norm = sum > 1.0 ? (float)sum : 1.f;
#pragma unroll
  for (int v = 0; v < 16; ++v)
    if (v < nv) {
      const float wv = w.p[v][i];
      if (mode == 0) {
        const double x = (double)wv / (double)norm * osem;
        w.p[v][i] = (float)(x != x ? x : fmin(1.0, x));
      } else {
        w.p[v][i] = java_min1(__fmul_rn((float)((double)wv / sum), (float)osem));
      }
    }
}

// k >= 0 rounded to `bits` significant bits, to nearest with ties to even
__device__ __forceinline__ long long round_sig(long long k, int bits) {
  const int nb = 64 - __clzll(k);
  if (nb <= bits) return k;
  const int sh = nb - bits;
  const long long low = k & ((1LL << sh) - 1), half = 1LL << (sh - 1);
  k -= low;
  if (low > half || (low == half && ((k >> sh) & 1))) k += 1LL << sh;
  return k;
}

// k * 2^e rounded once to float (|k| < 2^62), in integer operations only (a 64-bit integer
// conversion would take the FP64 pipe); false when the result is not a normal float
__device__ __forceinline__ bool scaled_float(long long k, int e, float& out) {
  if (k == 0) {
    out = 0.f;
    return true;
  }
  const unsigned sign = k < 0 ? 0x80000000u : 0u;
  const long long a = round_sig(k < 0 ? -k : k, 24);
  const int nb = 64 - __clzll(a);  // a = m 2^(nb - 24), m in [2^23, 2^24)
  const unsigned m = nb >= 24 ? (unsigned)(a >> (nb - 24)) : (unsigned)a << (24 - nb);
  const int ex = nb - 1 + e + 127;
  if (ex < 1 || ex > 254) return false;
  out = __uint_as_float(sign | ((unsigned)ex << 23) | (m & 0x7fffffu));
  return true;
}

// The reference's sequential double sum of the views' weights (0.0 + w_0 + w_1 + ...), as
// the float pair hi = (float)sum, lo = (float)(sum - hi), without FP64 arithmetic (GB300's FP64
// pipe would bound the kernel).  A positive float is m 2^s with a 24-bit integer m; aligned on
// the smallest s of the nonzero weights, every partial sum is an integer K, and the double
// addition's rounding is K rounded to 53 significant bits (ties to even), so the integers
// follow the double sum exactly.  false when that is not certain: a negative, infinite or NaN
// weight, exponents spread over more than 34 binades (the aligned sum would overflow 63 bits),
// or a result outside the normal float range; the caller then sums in double.
__device__ __forceinline__ bool exact_view_sum(const float* wv, int nv, float& hi, float& lo) {
  int emin = 1 << 20, emax = -(1 << 20);
#pragma unroll
  for (int v = 0; v < 16; ++v)
    if (v < nv) {
      const unsigned b = __float_as_uint(wv[v]);
      if (b & 0x80000000u) {
        if (b != 0x80000000u) return false;  // negative (-0 adds nothing)
        continue;
      }
      const int be = (int)(b >> 23);
      if (be == 255) return false;
      if (b == 0) continue;
      const int sv = (be ? be : 1) - 150;
      emin = min(emin, sv);
      emax = max(emax, sv);
    }
  if (emax < emin) {  // every weight zero
    hi = lo = 0.f;
    return true;
  }
  if (emax - emin > 34) return false;
  long long k = 0;
#pragma unroll
  for (int v = 0; v < 16; ++v)
    if (v < nv) {
      const unsigned b = __float_as_uint(wv[v]);
      if (b == 0u || b == 0x80000000u) continue;
      const int be = (int)(b >> 23);
      const long long m = (long long)((b & 0x7fffffu) | (be ? 0x800000u : 0u));
      k = round_sig(k + (m << (((be ? be : 1) - 150) - emin)), 53);
    }
  const long long khi = round_sig(k, 24);
  return scaled_float(khi, emin, hi) && scaled_float(k - khi, emin, lo);
}

struct Deferred {  // voxels left to the double pass
  long long* list;
  unsigned long long* count;
  unsigned long long cap;
};

// mode 0, VIRTUAL (NormalizingRandomAccess.get): w_v / (sum_w > 1 ? sum_w : 1), the sum in
// double and the normaliser stored as float, then min(1, w * osem) in double.  For osem == 1
// the float division is the result: the double quotient of two floats rounded to float is the
// correctly rounded float quotient.
// mode 1, PRECOMPUTED (WeightNormalizer.ApplyDirectly + ProcessForDeconvolution.adjustForOSEM):
// (float)(w_v / sum_w) with no guard on the sum (0 / 0 gives NaN where no view has weight, as
// in the reference), then min(1, w * (float)osem) in float.
// osem arrives as a float pair too (osem_hi + osem_lo == osem to ~48 bits).
// The view count is a template parameter: guards on a runtime count would still issue the
// instructions of all 16 view slots.
template <int NV>
__global__ void normalize_weights_kernel(WeightPtrs w, long long n, double osem, float osem_hi, float osem_lo,
                                         int mode, Deferred def) {
  constexpr int nv = NV;
  const FF os = {osem_hi, osem_lo};
  const bool unit = osem == 1.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float wv[16], out[16];
#pragma unroll
    for (int v = 0; v < 16; ++v)
      if (v < nv) wv[v] = w.p[v][i];
    float s_hi, s_lo;  // (float)sum_w and (float)(sum_w - s_hi)
    if (!exact_view_sum(wv, nv, s_hi, s_lo)) {
      double sum_d = 0.0;
#pragma unroll
      for (int v = 0; v < 16; ++v)
        if (v < nv) sum_d += (double)wv[v];
      s_hi = (float)sum_d;
      s_lo = (float)(sum_d - (double)s_hi);
    }
    bool certain = true;
    if (mode == 0) {
      // sum_w > 1 ? (float)sum_w : 1, NaN included (a NaN sum gives 1)
      const float norm = fmaxf(s_hi, 1.f);
#pragma unroll
      for (int v = 0; v < 16; ++v)
        if (v < nv) {
          float y;
          if (unit) {
            y = __fdiv_rn(wv[v], norm);
          } else {
            const FF q = ff_quotient(wv[v], FF{norm, 0.f});
            certain = !tiny(wv[v]) && !tiny(q.hi) && round_pair(ff_mul(q, os), y) && certain;
          }
          out[v] = java_min1(y);
        }
    } else {
      const FF sum = {s_hi, s_lo};
#pragma unroll
      for (int v = 0; v < 16; ++v)
        if (v < nv) {
          float x = 0.f;
          if (s_hi == 0.f) {  // a sum of floats is 0 or at least 2^-149 in magnitude
            x = __fdiv_rn(wv[v], 0.f);  // w / 0: NaN (0 / 0) or an infinity, as in double
          } else {
            certain = !tiny(wv[v]) && !tiny(s_hi) && round_pair(ff_quotient(wv[v], sum), x) && certain;
          }
          out[v] = java_min1(__fmul_rn(x, osem_hi));  // (float)osemspeedup: the float osem
        }
    }
    if (certain) {
#pragma unroll
      for (int v = 0; v < 16; ++v)
        if (v < nv) w.p[v][i] = out[v];
    } else {
      const unsigned m = __activemask();  // the lanes deferring a voxel in this step
      const int lane = threadIdx.x & 31;
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(def.count, (unsigned long long)__popc(m));
      base = __shfl_sync(m, base, leader);
      const unsigned long long slot = base + __popc(m & ((1u << lane) - 1u));
      if (slot < def.cap)
        def.list[slot] = i;
      else
        normalize_voxel_double(w, nv, i, osem, mode);  // list full: finish it here
    }
  }
}

__global__ void normalize_deferred_kernel(WeightPtrs w, int nv, double osem, int mode, Deferred def) {
  const unsigned long long cnt = *def.count;
  const unsigned long long m = cnt < def.cap ? cnt : def.cap;
  for (unsigned long long j = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; j < m;
       j += (unsigned long long)gridDim.x * blockDim.x)
    normalize_voxel_double(w, nv, def.list[j], osem, mode);
}

// WeightNormalizer's overlap statistics (WeightNormalizer.java:187-252): per voxel the number
// of views with weight > 0; the minimum over the volume and, per portion of
// FusionHelper.divideIntoPortions(n, P), the sum of the counts.  Each block walks one
// contiguous range, so a warp's 32 voxels lie in one portion except at the few portion
// borders; lane 0 keeps the running sum of its portion in a register.
template <int NV>
__global__ void weight_overlap_kernel(WeightPtrs w, long long n, long long chunk, int portions, long long span,
                                      unsigned long long* __restrict__ portion_sum, int* __restrict__ min_count) {
  constexpr int nv = NV;
  const long long lo = blockIdx.x * span;
  const long long hi = lo + span < n ? lo + span : n;
  const int lane = threadIdx.x & 31;
  int local_min = nv;
  int cur = -1;
  unsigned long long acc = 0;
  // portion of i = min(P - 1, i / chunk), followed incrementally from one 64-bit division:
  // p0 is the portion of the warp's first voxel, [p0 chunk, bnd) its range
  const long long first = lo + (threadIdx.x & ~31);
  int p0 = first < hi ? (int)min((long long)portions - 1, first / chunk) : 0;
  long long bnd = p0 == portions - 1 ? LLONG_MAX : (long long)(p0 + 1) * chunk;
  for (long long base = first; base < hi; base += blockDim.x) {
    const long long i = base + lane;
    int c = 0;
    if (i < hi) {
#pragma unroll
      for (int v = 0; v < 16; ++v)
        if (v < nv) c += w.p[v][i] > 0.f;
      local_min = min(local_min, c);
    }
    while (base >= bnd) {
      ++p0;
      bnd = p0 == portions - 1 ? LLONG_MAX : bnd + chunk;
    }
    const long long last = (base + 31 < hi ? base + 31 : hi - 1);
    if (last < bnd) {
      const unsigned s = __reduce_add_sync(0xffffffffu, (unsigned)c);
      if (lane == 0) {
        if (p0 != cur) {
          if (cur >= 0 && acc) atomicAdd(portion_sum + cur, acc);
          cur = p0;
          acc = 0;
        }
        acc += s;
      }
    } else if (i < hi && c) {
      int p = p0;
      for (long long b = bnd; i >= b;) {  // the warp spans at most 32 voxels
        ++p;
        b = p == portions - 1 ? LLONG_MAX : b + chunk;
      }
      atomicAdd(portion_sum + p, (unsigned long long)c);
    }
  }
  if (lane == 0 && cur >= 0 && acc) atomicAdd(portion_sum + cur, acc);
  const int m = __reduce_min_sync(0xffffffffu, local_min);
  if (lane == 0) atomicMin(min_count, m);
}

// f(std::integral_constant<int, nv>{}) for a view count 1..16
template <class F>
void with_view_count(int nv, F&& f) {
  switch (nv) {
#define MVD_NV_CASE(N) \
  case N:              \
    f(std::integral_constant<int, N>{}); \
    break;
    MVD_NV_CASE(1) MVD_NV_CASE(2) MVD_NV_CASE(3) MVD_NV_CASE(4) MVD_NV_CASE(5) MVD_NV_CASE(6) MVD_NV_CASE(7)
    MVD_NV_CASE(8) MVD_NV_CASE(9) MVD_NV_CASE(10) MVD_NV_CASE(11) MVD_NV_CASE(12) MVD_NV_CASE(13)
    MVD_NV_CASE(14) MVD_NV_CASE(15) MVD_NV_CASE(16)
#undef MVD_NV_CASE
    default:
      throw std::invalid_argument("1..16 views");
  }
}

int grid_n(long long n) {
  long long b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152LL * 32 ? 152LL * 32 : b));
}

bool g_lut_ready[64] = {};

void upload_lut(int dev) {
  if (dev < 64 && g_lut_ready[dev]) return;
  double lut[1001] = {};
  float2 pair[1001];
  // the reference's static block: d steps by 0.001 in double from 0 while d <= 1.0001, and
  // entry round(d * 1000) holds the value at the accumulated d (not exactly k / 1000)
  for (double d = 0; d <= 1.0001; d = d + 0.001)
    lut[(int)std::floor(d * 1000.0 + 0.5)] = (std::cos((1 - d) * M_PI) + 1) / 2;
  for (int k = 0; k <= 1000; ++k) {
    const float hi = (float)lut[k];
    pair[k] = make_float2(hi, (float)(lut[k] - (double)hi));
  }
  MVD_CHECK(cudaMemcpyToSymbol(g_blend_lut, lut, sizeof(lut)));
  MVD_CHECK(cudaMemcpyToSymbol(g_blend_pair, pair, sizeof(pair)));
  if (dev < 64) g_lut_ready[dev] = true;
}

bool invert_affine(const double* a, Affine& out) {
  // a: row-packed 3x4 [R | t] (view -> world); inverse = [R^-1 | -R^-1 t]
  const double r00 = a[0], r01 = a[1], r02 = a[2], r10 = a[4], r11 = a[5], r12 = a[6], r20 = a[8], r21 = a[9],
               r22 = a[10];
  const double det = r00 * (r11 * r22 - r12 * r21) - r01 * (r10 * r22 - r12 * r20) + r02 * (r10 * r21 - r11 * r20);
  if (!(std::fabs(det) > 0.0)) return false;
  double inv[9] = {(r11 * r22 - r12 * r21) / det, (r02 * r21 - r01 * r22) / det, (r01 * r12 - r02 * r11) / det,
                   (r12 * r20 - r10 * r22) / det, (r00 * r22 - r02 * r20) / det, (r02 * r10 - r00 * r12) / det,
                   (r10 * r21 - r11 * r20) / det, (r01 * r20 - r00 * r21) / det, (r00 * r11 - r01 * r10) / det};
  const double t[3] = {a[3], a[7], a[11]};
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) out.m[4 * r + c] = (float)inv[3 * r + c];
    out.m[4 * r + 3] = (float)-(inv[3 * r] * t[0] + inv[3 * r + 1] * t[1] + inv[3 * r + 2] * t[2]);
  }
  return true;
}

}  // namespace

extern "C" int mvd_transform_view(const float* view, const int* vd, const double* affine, const int* offset,
                                  const int* od, float* out_img, float* out_blend, const float* border,
                                  const float* blending, int devCUDA, void* stream) {
  try {
    set_last_error("");
    if (!view || !vd || !affine || !offset || !od || (!out_img && !out_blend)) {
      set_last_error("NULL argument");
      return MVD_ERR_ARG;
    }
    if (out_blend && (!border || !blending)) {
      set_last_error("blending weights need border and blending sizes");
      return MVD_ERR_ARG;
    }
    for (int d = 0; d < 3; ++d) {
      if (vd[d] < 1 || od[d] < 1) {
        set_last_error("sizes must be positive");
        return MVD_ERR_ARG;
      }
      if (out_blend && !(blending[d] > 0.f)) {
        set_last_error("blending sizes must be positive");
        return MVD_ERR_ARG;
      }
    }
    Affine inv;
    if (!invert_affine(affine, inv)) {
      set_last_error("the affine transform is singular");
      return MVD_ERR_ARG;
    }
    int count = 0;
    MVD_CHECK(cudaGetDeviceCount(&count));
    if (devCUDA < 0 || devCUDA >= count) {
      set_last_error("invalid CUDA device id");
      return MVD_ERR_ARG;
    }
    MVD_CHECK(cudaSetDevice(devCUDA));
    upload_lut(devCUDA);
    const float3 b = out_blend ? make_float3(border[0], border[1], border[2]) : make_float3(0.f, 0.f, 0.f);
    const float3 r = out_blend ? make_float3(blending[0], blending[1], blending[2]) : make_float3(1.f, 1.f, 1.f);
    if (od[2] > 65535 || od[1] > 8 * 65535) {
      set_last_error("output height above 524280 or depth above 65535");
      return MVD_ERR_ARG;
    }
    const bool narrow = (long long)vd[0] * vd[1] * vd[2] < (1LL << 31);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the warp runs along the output axis that moves the view position most along view x
    // (inv.m[0] and inv.m[2]: d(view x) / d(output x) and d(view x) / d(output z))
    if (std::fabs(inv.m[2]) > std::fabs(inv.m[0]) && od[1] <= 65535) {
      const dim3 grid((od[0] + 31) / 32, od[1], (od[2] + 31) / 32);
      (narrow ? transform_view_zfast_kernel<int> : transform_view_zfast_kernel<long long>)<<<grid, dim3(32, 8), 0,
                                                                                              s>>>(
          view, vd[0], vd[1], vd[2], inv, offset[0], offset[1], offset[2], od[0], od[1], od[2], out_img, out_blend, b,
          r);
    } else {
      const dim3 grid((od[0] + 31) / 32, (od[1] + 7) / 8, od[2]);
      (narrow ? transform_view_kernel<int> : transform_view_kernel<long long>)<<<grid, dim3(32, 8), 0, s>>>(
          view, vd[0], vd[1], vd[2], inv, offset[0], offset[1], offset[2], od[0], od[1], out_img, out_blend, b, r);
    }
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

extern "C" int mvd_normalize_weights(float* const* weights, int num_views, long long n, double osem, int mode,
                                     int devCUDA, void* stream) {
  try {
    set_last_error("");
    if (!weights || num_views < 1 || num_views > 16 || n < 0 || (mode != 0 && mode != 1)) {
      set_last_error("bad arguments (1..16 weight volumes, mode 0 or 1)");
      return MVD_ERR_ARG;
    }
    WeightPtrs wp{};
    for (int v = 0; v < num_views; ++v) {
      if (!weights[v]) {
        set_last_error("NULL weight volume");
        return MVD_ERR_ARG;
      }
      wp.p[v] = weights[v];
    }
    MVD_CHECK(cudaSetDevice(devCUDA));
    if (n == 0) return MVD_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const float osem_hi = (float)osem;
    const float osem_lo = (float)(osem - (double)osem_hi);
    // the deferred-voxel list, stream-ordered so that the call stays asynchronous
    Deferred def;
    def.cap = (unsigned long long)(n < (1LL << 22) ? n : (1LL << 22));
    void* buf = nullptr;
    MVD_CHECK(cudaMallocAsync(&buf, sizeof(unsigned long long) + def.cap * sizeof(long long), s));
    def.count = static_cast<unsigned long long*>(buf);
    def.list = reinterpret_cast<long long*>(def.count + 1);
    MVD_CHECK(cudaMemsetAsync(def.count, 0, sizeof(unsigned long long), s));
    with_view_count(num_views, [&](auto nv) {
      normalize_weights_kernel<decltype(nv)::value><<<grid_n(n), 256, 0, s>>>(wp, n, osem, osem_hi, osem_lo, mode, def);
    });
    MVD_CHECK(cudaGetLastError());
    count_launch();
    normalize_deferred_kernel<<<152 * 4, 256, 0, s>>>(wp, num_views, osem, mode, def);
    MVD_CHECK(cudaGetLastError());
    count_launch();
    MVD_CHECK(cudaFreeAsync(buf, s));
    return MVD_OK;
  } catch (const CudaError& e) {
    set_last_error(e.what());
    return MVD_ERR_CUDA;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return MVD_ERR_INTERNAL;
  }
}

extern "C" int mvd_weight_overlap(const float* const* weights, int num_views, long long n, int num_portions,
                                  int* min_views, double* avg_views, int devCUDA, void* stream) {
  try {
    set_last_error("");
    if (!weights || num_views < 1 || num_views > 16 || n < 1 || num_portions < 1 || num_portions > 65536 ||
        (long long)num_portions > n || !min_views || !avg_views) {
      set_last_error("bad arguments (1..16 weight volumes, 1 <= num_portions <= min(n, 65536))");
      return MVD_ERR_ARG;
    }
    WeightPtrs wp{};
    for (int v = 0; v < num_views; ++v) {
      if (!weights[v]) {
        set_last_error("NULL weight volume");
        return MVD_ERR_ARG;
      }
      wp.p[v] = const_cast<float*>(weights[v]);
    }
    MVD_CHECK(cudaSetDevice(devCUDA));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // device scratch: the portion sums, then the minimum
    const size_t bytes = (size_t)num_portions * sizeof(unsigned long long) + sizeof(int);
    DevBuf scratch;
    scratch.alloc(bytes);
    unsigned long long* d_sum = scratch.as<unsigned long long>();
    int* d_min = reinterpret_cast<int*>(d_sum + num_portions);
    MVD_CHECK(cudaMemsetAsync(d_sum, 0, (size_t)num_portions * sizeof(unsigned long long), s));
    MVD_CHECK(cudaMemcpyAsync(d_min, &num_views, sizeof(int), cudaMemcpyHostToDevice, s));
    const int grid = grid_n(n);
    long long span = (n + grid - 1) / grid;
    span = (span + 31) / 32 * 32;
    const long long chunk = n / num_portions;
    with_view_count(num_views, [&](auto nv) {
      weight_overlap_kernel<decltype(nv)::value><<<grid, 256, 0, s>>>(wp, n, chunk, num_portions, span, d_sum, d_min);
    });
    MVD_CHECK(cudaGetLastError());
    count_launch();
    std::vector<unsigned long long> sums(num_portions);
    int mn = 0;
    MVD_CHECK(cudaMemcpyAsync(sums.data(), d_sum, sums.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    MVD_CHECK(cudaMemcpyAsync(&mn, d_min, sizeof(int), cudaMemcpyDeviceToHost, s));
    MVD_CHECK(cudaStreamSynchronize(s));
    // the reference averages the per-portion averages (WeightNormalizer.java:98-106)
    double avg = 0.0;
    for (int p = 0; p < num_portions; ++p) {
      const long long loop = p == num_portions - 1 ? chunk + n % num_portions : chunk;
      avg += (double)sums[p] / (double)loop;
    }
    *min_views = mn;
    *avg_views = avg / num_portions;
    return MVD_OK;
  } catch (const CudaError& e) {
    set_last_error(e.what());
    return MVD_ERR_CUDA;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return MVD_ERR_INTERNAL;
  }
}
