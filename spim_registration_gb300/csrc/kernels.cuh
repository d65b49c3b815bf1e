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

constexpr int kThreads = 512;    // threads per CTA of the plane kernels
constexpr int kZThreads = 256;   // threads per CTA of the z-pencil kernel
constexpr int kPlaneCap = 14336; // complex values of one shared-memory buffer (two are used)
constexpr int kZChunk = 16;      // pencils per z-pass CTA (16 complex = one 128-byte line)
constexpr int kZPitch = kZChunk + 1;

// Row pitch (complex values, odd) that holds a half-spectrum row of px = M + 1 values and
// the skewed layout i + i/16 of a length-M row between the first two row stages.
__host__ __device__ inline int row_pitch(int M) {
  int p = M + 1;
  const int skew = M + (M - 1) / 16 + 1;
  if (skew > p) p = skew;
  return (p & 1) ? p : p + 1;
}

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
// load / store functors of the first and last FFT stages
// ------------------------------------------------------------------------------------------
// row element i of a row stored with the skew i + i/16 (used between row stages 0 and 1)
struct SmemRowSkew {
  float2* p;
  int pitch;
  __device__ __forceinline__ float2 operator()(int batch, int i) const { return p[batch * pitch + i + (i >> 4)]; }
  __device__ __forceinline__ void operator()(int batch, int i, float2 v) const { p[batch * pitch + i + (i >> 4)] = v; }
};

template <class Gather>
struct RowGather {  // packed pair (x[2n], x[2n+1]) of tile row `batch`, gathered from the volume
  Gather g;
  int ox, oy, gz;
  __device__ __forceinline__ float2 operator()(int batch, int n) const {
    const int gx = ox + 2 * n, gy = oy + batch;
    return make_float2(g(gx, gy, gz), g(gx + 1, gy, gz));
  }
};

struct SpecSliceLoad {  // spectrum slice [y][kx]: batch = kx, i = y
  const float2* p;
  int px;
  __device__ __forceinline__ float2 operator()(int batch, int i) const { return __ldg(p + i * px + batch); }
};

struct SpecSliceStore {
  float2* p;
  int px;
  __device__ __forceinline__ void operator()(int batch, int i, float2 v) const { p[i * px + batch] = v; }
};

struct PencilRef {  // pencil element: batch = pencil in the chunk, i = z
  float2* p;
  long long plane;
  __device__ __forceinline__ float2 operator()(int batch, int i) const { return p[i * plane + batch]; }
  __device__ __forceinline__ void operator()(int batch, int i, float2 v) const { p[i * plane + batch] = v; }
};

struct PencilScaledStore {
  float2* p;
  long long plane;
  float scale;
  __device__ __forceinline__ void operator()(int batch, int i, float2 v) const { p[i * plane + batch] = cscale(v, scale); }
};

struct OtfMul {
  const float2* p;
  long long plane;
  __device__ __forceinline__ float2 operator()(int batch, int k, float2 v) const {
    return cmul(v, __ldg(p + k * plane + batch));
  }
};

template <class Epi>
struct RowEpilogue {  // last inverse x stage: complex n of effective row `batch` = reals 2n, 2n+1
  Epi* epi;
  long long row0;     // global index of tile-local (x = 0, y = hy, z) in the volume
  long long ystride;  // global stride of one row
  int hx, ex;
  __device__ __forceinline__ void operator()(int batch, int n, float2 v) const {
    const long long g = row0 + batch * ystride;
    const int x0 = 2 * n - hx;
    if (x0 >= 0 && x0 < ex) (*epi)(g + x0, v.x);
    if (x0 + 1 >= 0 && x0 + 1 < ex) (*epi)(g + x0 + 1, v.y);
  }
};

// Stage dispatch over the shared-memory layouts: `skew_in` / `skew_out` select the skewed
// row layout (i + i/16) for the buffer read / written.
template <bool INV, bool JFAST, class LD>
__device__ __forceinline__ void stage_to_smem(int R, int n, int Ns, int count, const float2* tw, const LD& ld,
                                              float2* dst, int es, int bs, bool skew_out) {
  if (skew_out)
    stage<INV, JFAST>(R, n, Ns, count, tw, ld, SmemRowSkew{dst, bs});
  else
    stage<INV, JFAST>(R, n, Ns, count, tw, ld, SmemRef{dst, es, bs});
}

template <bool INV, bool JFAST, class ST>
__device__ __forceinline__ void stage_from_smem(int R, int n, int Ns, int count, const float2* tw, float2* src,
                                                int es, int bs, bool skew_in, const ST& st) {
  if (skew_in)
    stage<INV, JFAST>(R, n, Ns, count, tw, SmemRowSkew{src, bs}, st);
  else
    stage<INV, JFAST>(R, n, Ns, count, tw, SmemRef{src, es, bs}, st);
}

// All stages of one transform with the result left in shared memory: on return (after a
// barrier) `cur` holds it in the plain layout.  Stage 0 loads with ld0 (global memory or
// `cur`) and every stage writes the other buffer.  ROWS (row transforms, es == 1): j-fastest
// butterflies and the skewed layout between stages 0 and 1.
template <bool INV, bool ROWS, class LD0>
__device__ __forceinline__ void run_transform_smem(const FftPlan* __restrict__ p, int count, const LD0& ld0,
                                                   float2*& cur, float2*& oth, int es, int bs) {
  const int n = __ldg(&p->n);
  const int ns = __ldg(&p->nstages);
  const float2* tw = p->tw;
  int Ns = 1;
  for (int s = 0; s < ns; ++s) {
    const int R = __ldg(&p->radix[s]);
    const bool skew_out = ROWS && s == 0 && ns > 1;
    if (s == 0) {
      stage_to_smem<INV, ROWS>(R, n, Ns, count, tw, ld0, oth, es, bs, skew_out);
    } else {
      if (ROWS && s == 1)
        stage<INV, ROWS>(R, n, Ns, count, tw, SmemRowSkew{cur, bs}, SmemRef{oth, es, bs});
      else
        stage<INV, ROWS>(R, n, Ns, count, tw, SmemRef{cur, es, bs}, SmemRef{oth, es, bs});
    }
    __syncthreads();
    float2* t = cur;
    cur = oth;
    oth = t;
    Ns *= R;
  }
}

// All stages of one transform with the last stage storing through `stl` (global memory or an
// epilogue).  Stage 0 loads with ld0; the exchanges in between alternate the two buffers.
template <bool INV, bool ROWS, class LD0, class STL>
__device__ __forceinline__ void run_transform_to(const FftPlan* __restrict__ p, int count, const LD0& ld0,
                                                 const STL& stl, float2*& cur, float2*& oth, int es, int bs) {
  const int n = __ldg(&p->n);
  const int ns = __ldg(&p->nstages);
  const float2* tw = p->tw;
  if (ns == 1) {
    stage<INV, ROWS>(__ldg(&p->radix[0]), n, 1, count, tw, ld0, stl);
    return;
  }
  int Ns = 1;
  for (int s = 0; s < ns; ++s) {
    const int R = __ldg(&p->radix[s]);
    const bool skew_in = ROWS && s == 1;
    if (s == ns - 1) {
      stage_from_smem<INV, ROWS>(R, n, Ns, count, tw, cur, es, bs, skew_in, stl);
    } else {
      if (s == 0)
        stage_to_smem<INV, ROWS>(R, n, Ns, count, tw, ld0, oth, es, bs, ROWS);
      else if (skew_in)
        stage<INV, ROWS>(R, n, Ns, count, tw, SmemRowSkew{cur, bs}, SmemRef{oth, es, bs});
      else
        stage<INV, ROWS>(R, n, Ns, count, tw, SmemRef{cur, es, bs}, SmemRef{oth, es, bs});
      __syncthreads();
      float2* t = cur;
      cur = oth;
      oth = t;
    }
    Ns *= R;
  }
}

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
  float2* cur = sm;
  float2* oth = sm + t.ty * t.pitch;
  // x: R2C of every row (packed pairs gathered straight from the volume)
  RowGather<Gather> ld0{gather, t.ox, t.oy, t.oz + z};
  const FftPlan* pxp = plans + t.plan_x;
  run_transform_smem<false, true>(pxp, t.ty, ld0, cur, oth, 1, t.pitch);
  r2c_post(cur, t.ty, M, t.pitch, pxp->tw_r2c);
  __syncthreads();
  // y: C2C of every column, last stage straight to the spectrum slice
  SpecSliceStore st{spec + t.spec_off + (long long)z * t.ty * t.px, t.px};
  run_transform_to<false, false>(plans + t.plan_y, t.px, SmemRef{cur, t.pitch, 1}, st, cur, oth, t.pitch, 1);
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
  float2* cur = sm;
  float2* oth = sm + t.ty * t.pitch;
  // y: inverse C2C of every column, first stage straight from the spectrum slice
  SpecSliceLoad ld{spec + t.spec_off + (long long)z * t.ty * t.px, t.px};
  run_transform_smem<true, false>(plans + t.plan_y, t.px, ld, cur, oth, t.pitch, 1);
  // only the effective rows go on: C2R pre-step and the inverse x transform
  float2* rows = cur + t.hy * t.pitch;
  float2* rows_oth = oth + t.hy * t.pitch;
  c2r_pre(rows, t.ey, M, t.pitch, plans[t.plan_x].tw_r2c);
  __syncthreads();
  const long long gz = t.oz + z;
  RowEpilogue<Epi> st{&epi, (gz * epi.ny + (t.oy + t.hy)) * (long long)epi.nx + t.ox + t.hx, (long long)epi.nx,
                      t.hx, t.ex};
  epi.acc_init();
  run_transform_to<true, true>(plans + t.plan_x, t.ey, SmemRef{rows, 1, t.pitch}, st, rows, rows_oth, 1, t.pitch);
  epi.finish();
}

// MODE 0: forward z, multiply by the OTF, inverse z.  MODE 1: forward z and scale (OTF build).
template <int MODE>
__global__ void __launch_bounds__(kZThreads)
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
  PencilRef g{spec + t.spec_off + p0, plane};
  const int n = __ldg(&pz->n);
  const int ns = __ldg(&pz->nstages);
  const float2* tw = pz->tw;
  if (MODE == 1) {
    run_transform_to<false, false>(pz, count, g, PencilScaledStore{g.p, plane, scale}, cur, oth, kZPitch, 1);
    return;
  }
  OtfMul mul{otf + t.otf_off + p0, plane};
  if (ns == 1) {
    zmid(__ldg(&pz->radix[0]), n, count, tw, g, mul, g);
    return;
  }
  // forward stages 0 .. ns-2
  int Ns = 1;
  for (int s = 0; s < ns - 1; ++s) {
    const int R = __ldg(&pz->radix[s]);
    if (s == 0) {
      stage<false, false>(R, n, Ns, count, tw, g, SmemRef{cur, kZPitch, 1});
    } else {
      stage<false, false>(R, n, Ns, count, tw, SmemRef{cur, kZPitch, 1}, SmemRef{oth, kZPitch, 1});
      float2* tmp = cur;
      cur = oth;
      oth = tmp;
    }
    __syncthreads();
    Ns *= R;
  }
  // forward last stage, product with the OTF, inverse first stage
  zmid(__ldg(&pz->radix[ns - 1]), n, count, tw, SmemRef{cur, kZPitch, 1}, mul, SmemRef{oth, kZPitch, 1});
  __syncthreads();
  {
    float2* tmp = cur;
    cur = oth;
    oth = tmp;
  }
  // inverse stages 1 .. ns-1 use the radices in reverse order
  Ns = __ldg(&pz->radix[ns - 1]);
  for (int i = 1; i < ns; ++i) {
    const int R = __ldg(&pz->radix[ns - 1 - i]);
    if (i == ns - 1) {
      stage<true, false>(R, n, Ns, count, tw, SmemRef{cur, kZPitch, 1}, g);
    } else {
      stage<true, false>(R, n, Ns, count, tw, SmemRef{cur, kZPitch, 1}, SmemRef{oth, kZPitch, 1});
      __syncthreads();
      float2* tmp = cur;
      cur = oth;
      oth = tmp;
    }
    Ns *= R;
  }
}

}  // namespace mvd
