// Tiled 3D FFT convolution kernels (sm_103a) for the multiview deconvolution path.
//
// A convolution of a volume with an odd-sized kernel is computed by overlap-save over tiles:
// tile t covers global coordinates [o, o + T) per axis (o = effective offset - k/2), is
// transformed as a circular 3D FFT of size T, multiplied by the kernel's spectrum (the OTF)
// and inverted; its effective region [k/2, k/2 + E) is exact linear convolution of the
// extended volume and is what the epilogue consumes.  This is the reference's block scheme
// (BlockGeneratorFixedSizePrecise.java:46-122, Block.java:134-379) with the FFT done on the
// GPU and the copy-in / paste-out fused into the first and last pass.
//
// Three passes per convolution, all driven by work-item tables so that every tile of every
// shape runs in the same launch:
//   plane_fwd : gather a z-slice of the tile (with the out-of-bounds rule), R2C along x,
//               C2C along y, store the half-spectrum slice  [z][y][kx] (kx fastest);
//   zpass     : for 32 consecutive (y, kx) pencils: C2C along z, multiply by the OTF,
//               inverse C2C along z (or, for OTF preparation, forward only and scale);
//   plane_inv : for an effective z-slice: inverse C2C along y, C2R along x, epilogue over
//               the effective (x, y) region (store / quotient / multiplicative update).
#pragma once
#include "fft_device.cuh"

namespace mvd {

constexpr int kThreads = 512;    // threads per CTA of the FFT kernels
constexpr int kPlaneCap = 14336; // complex values of one shared-memory buffer (two are used)
constexpr int kZChunk = 32;      // pencils per z-pass CTA
constexpr int kZPitch = kZChunk + 1;

struct TileDesc {
  int tx, ty, tz;        // FFT size of the tile
  int px;                // tx / 2 + 1 (half-spectrum row length)
  int pitch;             // shared-memory row pitch in complex values (odd, >= px)
  int ox, oy, oz;        // global coordinate of tile-local (0,0,0)
  int hx, hy, hz;        // tile-local start of the effective region (kernel half sizes)
  int ex, ey, ez;        // effective region size (clipped to the volume)
  int plan_x, plan_y, plan_z;  // plan-table indices (plan_x has length tx/2)
  int pad_;
  long long spec_off;    // tile spectrum offset (complex elements)
  long long otf_off;     // tile OTF offset (complex elements)
};

struct VolumeRef {
  const float* data;
  int nx, ny, nz;
};

// ------------------------------------------------------------------------------------------
// out-of-bounds rules of the two convolutions of an iteration
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ int mirror_single(int i, int n) {
  // Views.extendMirrorSingle: -1 -> 1, n -> n-2, period 2n-2
  if (i >= 0 && i < n) return i;
  if (n == 1) return 0;
  const int period = 2 * n - 2;
  int m = i % period;
  if (m < 0) m += period;
  return m < n ? m : period - m;
}

struct GatherMirror {  // psi extended mirror-single (MVDeconFFTThreads.java:44,78)
  VolumeRef v;
  __device__ __forceinline__ float operator()(int gx, int gy, int gz) const {
    gx = mirror_single(gx, v.nx);
    gy = mirror_single(gy, v.ny);
    gz = mirror_single(gz, v.nz);
    return __ldg(v.data + ((long long)gz * v.ny + gy) * v.nx + gx);
  }
};

struct GatherValue {  // quotient extended with a constant (value 1: MVDeconFFTThreads.java:63,103)
  VolumeRef v;
  float value;
  __device__ __forceinline__ float operator()(int gx, int gy, int gz) const {
    if (gx < 0 || gy < 0 || gz < 0 || gx >= v.nx || gy >= v.ny || gz >= v.nz) return value;
    return __ldg(v.data + ((long long)gz * v.ny + gy) * v.nx + gx);
  }
};

// ------------------------------------------------------------------------------------------
// epilogues of the inverse plane pass: called once per effective voxel, then finish()
// ------------------------------------------------------------------------------------------
struct EpiStore {
  float* out;
  int nx, ny;
  __device__ __forceinline__ void acc_init() {}
  __device__ __forceinline__ void operator()(long long g, float v) { out[g] = v; }
  __device__ __forceinline__ void finish() {}
};

// MVDeconvolution.computeQuotient (MVDeconvolution.java:494-546): img > 0 ? img / blurred : 1
struct EpiQuotient {
  const float* img;
  float* q;
  int nx, ny;
  __device__ __forceinline__ void acc_init() {}
  __device__ __forceinline__ void operator()(long long g, float blurred) {
    const float i = __ldg(img + g);
    q[g] = i > 0.f ? __fdiv_rn(i, blurred) : 1.f;
  }
  __device__ __forceinline__ void finish() {}
};

// MVDeconvolution.computeFinalValues / computeNextValue / tikhonov (:603-726).  The reference
// evaluates tikhonov in double and rounds to float; here the algebraically equal form
// 2v / (sqrt(1 + 2 lambda v) + 1) is evaluated in float (no cancellation, within a few ulp).
// Statistics (sum and max of |change|) are accumulated in FP64.
struct EpiUpdate {
  float* psi;
  const float* weight;
  float lambda;
  double* stat_sum;    // += sum |change| (FP64)
  unsigned* stat_max;  // max |change| as float bits (changes are >= 0)
  int nx, ny;
  float acc_sum;
  float acc_max;
  __device__ __forceinline__ void acc_init() {
    acc_sum = 0.f;
    acc_max = 0.f;
  }
  __device__ __forceinline__ void operator()(long long g, float integral) {
    const float last = psi[g];
    const float value = __fmul_rn(last, integral);
    float adjusted;
    if (value > 0.f) {
      if (lambda > 0.f && !isinf(value)) {
        const float r = __fsqrt_rn(__fadd_rn(1.f, __fmul_rn(2.f * lambda, value)));
        adjusted = __fdiv_rn(__fmul_rn(2.f, value), __fadd_rn(r, 1.f));
      } else {
        adjusted = value;
      }
    } else {
      adjusted = 1e-4f;
    }
    const float next = isnan(adjusted) ? 1e-4f : fmaxf(1e-4f, adjusted);
    const float w = __ldg(weight + g);
    const float out = __fadd_rn(last, __fmul_rn(__fsub_rn(next, last), w));
    psi[g] = out;
    const float change = fabsf(__fsub_rn(out, last));
    acc_sum += change;
    acc_max = fmaxf(acc_max, change);
  }
  __device__ __forceinline__ void finish() {
    // FP64 block reduction of the per-thread partials, one atomic per CTA
    __shared__ double red_sum[32];
    __shared__ float red_max[32];
    double sum = (double)acc_sum;
    float mx = acc_max;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sum += __shfl_xor_sync(0xffffffffu, sum, o);
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
      red_sum[warp] = sum;
      red_max[warp] = mx;
    }
    __syncthreads();
    if (warp == 0) {
      const int nw = blockDim.x >> 5;
      sum = lane < nw ? red_sum[lane] : 0.0;
      mx = lane < nw ? red_max[lane] : 0.f;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      }
      if (lane == 0) {
        atomicAdd(stat_sum, sum);
        atomicMax(stat_max, __float_as_uint(mx));
      }
    }
  }
};

// ------------------------------------------------------------------------------------------
// kernels (templated on gather / epilogue; instantiated in engine.cu)
// ------------------------------------------------------------------------------------------
template <class Gather>
__global__ void __launch_bounds__(kThreads, 1)
plane_fwd_kernel(const TileDesc* __restrict__ tiles, const int2* __restrict__ items,
                 const FftPlan* __restrict__ plans, float2* __restrict__ spec, Gather gather) {
  extern __shared__ float2 sm[];
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int z = it.y;
  const int M = t.tx / 2;
  const FftPlan* px_plan = plans + t.plan_x;
  const FftPlan* py_plan = plans + t.plan_y;
  float2* cur = sm;
  float2* oth = sm + t.ty * t.pitch;
  float* smf = reinterpret_cast<float*>(cur);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int gz = t.oz + z;
  for (int y = warp; y < t.ty; y += nwarps) {
    const int gy = t.oy + y;
    float* row = smf + 2 * y * t.pitch;
    for (int x = lane; x < t.tx; x += 32) row[x] = gather(t.ox + x, gy, gz);
  }
  __syncthreads();
  block_fft<false>(cur, oth, px_plan, t.ty, 1, t.pitch);
  r2c_post(cur, t.ty, M, t.pitch, px_plan->tw_r2c);
  block_fft<false>(cur, oth, py_plan, t.px, t.pitch, 1);
  float2* dst = spec + t.spec_off + (long long)z * t.ty * t.px;
  for (int y = warp; y < t.ty; y += nwarps) {
    const float2* row = cur + y * t.pitch;
    for (int x = lane; x < t.px; x += 32) dst[y * t.px + x] = row[x];
  }
}

template <class Epi>
__global__ void __launch_bounds__(kThreads, 1)
plane_inv_kernel(const TileDesc* __restrict__ tiles, const int2* __restrict__ items,
                 const FftPlan* __restrict__ plans, const float2* __restrict__ spec, Epi epi) {
  extern __shared__ float2 sm[];
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int z = it.y;  // tile-local slice, inside the effective range
  const int M = t.tx / 2;
  const FftPlan* px_plan = plans + t.plan_x;
  const FftPlan* py_plan = plans + t.plan_y;
  float2* cur = sm;
  float2* oth = sm + t.ty * t.pitch;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const float2* src = spec + t.spec_off + (long long)z * t.ty * t.px;
  for (int y = warp; y < t.ty; y += nwarps) {
    float2* row = cur + y * t.pitch;
    for (int x = lane; x < t.px; x += 32) row[x] = __ldg(src + y * t.px + x);
  }
  __syncthreads();
  block_fft<true>(cur, oth, py_plan, t.px, t.pitch, 1);
  c2r_pre(cur, t.ty, M, t.pitch, px_plan->tw_r2c);
  block_fft<true>(cur, oth, px_plan, t.ty, 1, t.pitch);
  const float* smf = reinterpret_cast<const float*>(cur);
  const long long gz = t.oz + z;
  epi.acc_init();
  for (int y = warp; y < t.ey; y += nwarps) {
    const int ly = t.hy + y;
    const long long grow = (gz * epi.ny + (t.oy + ly)) * (long long)epi.nx + t.ox;
    const float* row = smf + 2 * ly * t.pitch;
    for (int x = lane; x < t.ex; x += 32) epi(grow + t.hx + x, row[t.hx + x]);
  }
  epi.finish();
}

// MODE 0: forward z, multiply by OTF, inverse z.  MODE 1: forward z and scale (OTF build).
template <int MODE>
__global__ void __launch_bounds__(kThreads, 1)
zpass_kernel(const TileDesc* __restrict__ tiles, const int2* __restrict__ items,
             const FftPlan* __restrict__ plans, float2* __restrict__ spec,
             const float2* __restrict__ otf, float scale) {
  extern __shared__ float2 sm[];
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int p0 = it.y;
  const long long plane = (long long)t.ty * t.px;
  const int count = min(kZChunk, (int)(plane - p0));
  const FftPlan* pz = plans + t.plan_z;
  float2* cur = sm;
  float2* oth = sm + t.tz * kZPitch;
  float2* base = spec + t.spec_off + p0;
  for (int i = threadIdx.x; i < t.tz * kZChunk; i += blockDim.x) {
    const int z = i / kZChunk, c = i % kZChunk;
    if (c < count) cur[z * kZPitch + c] = base[z * plane + c];
  }
  __syncthreads();
  block_fft<false>(cur, oth, pz, count, kZPitch, 1);
  if (MODE == 0) {
    const float2* o = otf + t.otf_off + p0;
    for (int i = threadIdx.x; i < t.tz * kZChunk; i += blockDim.x) {
      const int z = i / kZChunk, c = i % kZChunk;
      if (c < count) cur[z * kZPitch + c] = cmul(cur[z * kZPitch + c], __ldg(o + z * plane + c));
    }
    __syncthreads();
    block_fft<true>(cur, oth, pz, count, kZPitch, 1);
  }
  for (int i = threadIdx.x; i < t.tz * kZChunk; i += blockDim.x) {
    const int z = i / kZChunk, c = i % kZChunk;
    if (c < count) {
      float2 v = cur[z * kZPitch + c];
      if (MODE == 1) v = cscale(v, scale);
      base[z * plane + c] = v;
    }
  }
}

}  // namespace mvd
