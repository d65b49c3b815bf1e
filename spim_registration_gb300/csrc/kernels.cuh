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
//   plane_fwd : gather a z-slice of the tile (with the out-of-bounds rule), R2C along x (a
//               half-length complex FFT of packed pairs; the real-spectrum step is folded
//               into the first y stage's loads), C2C along y, store the half-spectrum slice
//               [z][y][kx] (kx fastest);
//   zpass     : for 32 consecutive (y, kx) pencils: C2C along z, multiply by the OTF,
//               inverse C2C along z (or, for OTF preparation, forward only and scale);
//   plane_inv : for an effective z-slice: inverse C2C along y, C2R along x of the effective
//               rows only (the half-spectrum step folded into the first x stage's loads),
//               epilogue over the effective (x, y) region (store / quotient / update / NLL).
#pragma once
#include <cuda.h>  // CUtensorMap

#include "fft_device.cuh"

namespace mvd {

// Tensor maps of the volumes an epilogue reads, with a box of one effective slice of a tile
// (x start rounded down to 16 bytes): the inverse pass prefetches them into L2 at its start,
// so the epilogue's loads, issued after the inverse FFT stages, find them there.
struct EpiBoxes {
  CUtensorMap map[2];
  int count;
};

// Box width (floats) of a volume slice's L2 prefetch: a tile row of TX values at any x offset in
// [0, 4) from the 16-byte boundary the box starts on, rounded up to 16 bytes.
__host__ __device__ constexpr int prefetch_box_width(int TX) { return (TX + 3 + 3) / 4 * 4; }

__device__ __forceinline__ void prefetch_box_l2(const CUtensorMap* map, int x, int y, int z) {
  asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(z)
               : "memory");
}


constexpr int kThreads = 384;    // threads per CTA of the plane kernels (two CTAs per SM: 24 warps)
constexpr int kZThreads = 256;   // threads per CTA of the z-pencil kernel
constexpr int kPlaneCap = 14336; // complex values of one shared-memory buffer (two are used)
constexpr int kPlaneCapDefault = 7168;  // planner default: two CTAs per SM (measured faster)
constexpr int kZChunk = 16;      // pencils per z-pass CTA (16 complex = one 128-byte line)
constexpr int kZPitch = kZChunk + 1;
constexpr int kZWideChunk = 32;  // pencils per CTA of the in-place compiled z pass (256-byte rows)

// Row pitch (complex values, odd) that holds a half-spectrum row of px = M + 1 values and
// the skewed layout i + i/16 of a length-M row between the first two row stages.
__host__ __device__ constexpr int row_pitch(int M) {
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

// Each gather resolves a row once (row(gy, gz)) and then reads x positions of that row.
struct GatherMirror {  // psi extended mirror-single (MVDeconFFTThreads.java:44,78)
  VolumeRef v;
  struct Row {
    const float* p;
    int nx;
    __device__ __forceinline__ float operator()(int gx) const { return __ldg(p + mirror_single(gx, nx)); }
  };
  __device__ __forceinline__ Row row(int gy, int gz) const {
    return Row{v.data + ((long long)mirror_single(gz, v.nz) * v.ny + mirror_single(gy, v.ny)) * v.nx, v.nx};
  }
  __device__ __forceinline__ float operator()(int gx, int gy, int gz) const { return row(gy, gz)(gx); }
  // for slice copies: the volume slice holding slice gz, and the (x, y) region read as is
  __device__ __forceinline__ bool slice_source(int gz, int& zsrc) const {
    zsrc = mirror_single(gz, v.nz);
    return true;
  }
  __device__ __forceinline__ void region(int& x0, int& x1, int& y0, int& y1) const {
    x0 = 0; x1 = v.nx; y0 = 0; y1 = v.ny;
  }
  // whether every value of slice gz is one constant (never: the mirror reads the volume)
  __device__ __forceinline__ bool constant_slice(int, float&) const { return false; }
};

struct GatherValue {  // quotient extended with a constant (value 1: MVDeconFFTThreads.java:63,103)
  VolumeRef v;
  float value;
  int lo[3], hi[3];  // the data box (x, y, z): `value` outside it
  __host__ __device__ static GatherValue full(const float* data, int nx, int ny, int nz, float value) {
    return box(data, nx, ny, nz, value, 0, 0, 0, nx, ny, nz);
  }
  __host__ __device__ static GatherValue box(const float* data, int nx, int ny, int nz, float value, int x0, int y0,
                                             int z0, int x1, int y1, int z1) {
    GatherValue g;
    g.v = VolumeRef{data, nx, ny, nz};
    g.value = value;
    g.lo[0] = x0; g.lo[1] = y0; g.lo[2] = z0;
    g.hi[0] = x1; g.hi[1] = y1; g.hi[2] = z1;
    return g;
  }
  struct Row {
    const float* p;  // nullptr: the whole row is outside the box
    int x0, x1;
    float value;
    __device__ __forceinline__ float operator()(int gx) const {
      return (p && gx >= x0 && gx < x1) ? __ldg(p + gx) : value;
    }
  };
  __device__ __forceinline__ Row row(int gy, int gz) const {
    const bool in = gy >= lo[1] && gz >= lo[2] && gy < hi[1] && gz < hi[2];
    return Row{in ? v.data + ((long long)gz * v.ny + gy) * v.nx : nullptr, lo[0], hi[0], value};
  }
  __device__ __forceinline__ float operator()(int gx, int gy, int gz) const { return row(gy, gz)(gx); }
  // for slice copies: false when slice gz lies outside the data box (all of it is `value`)
  __device__ __forceinline__ bool slice_source(int gz, int& zsrc) const {
    zsrc = gz;
    return gz >= lo[2] && gz < hi[2];
  }
  __device__ __forceinline__ void region(int& x0, int& x1, int& y0, int& y1) const {
    x0 = lo[0]; x1 = hi[0]; y0 = lo[1]; y1 = hi[1];
  }
  // whether every value of slice gz is one constant: a slice outside the data box is `value`
  __device__ __forceinline__ bool constant_slice(int gz, float& c) const {
    c = value;
    return gz < lo[2] || gz >= hi[2];
  }
};

// The half-spectrum slice [y][kx] of a constant slice c of tx x ty reals: the DC term c tx ty,
// zero elsewhere (the forward transform is unnormalised).  The second convolution's input is
// extended with the value 1 outside the view's data box, so the slices of a tile's z halo that
// lie outside the box take this path instead of a gather and two transforms.
__device__ __forceinline__ void constant_spectrum_slice(float2* p, int tx, int ty, int px, float c) {
  const int n = ty * px;
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = make_float2(i == 0 ? c * (float)tx * (float)ty : 0.f, 0.f);
}

// ------------------------------------------------------------------------------------------
// epilogues of the inverse plane pass.  apply<K>(g0, off, val, ok) handles K voxels of one row
// (global index g0 + off[i], value val[i], in the effective region if ok[i]): all loads are
// issued before any store.  finish() ends the CTA's work (statistics).
// ------------------------------------------------------------------------------------------
struct EpiStore {
  float* out;
  int nx, ny;
  int inputs(const float** p) const { return 0; }  // volumes the epilogue reads (for L2 prefetch)
  __device__ __forceinline__ void acc_init() {}
  __device__ __forceinline__ void operator()(long long g, float v) { out[g] = v; }
  template <int K>
  __device__ __forceinline__ void apply(long long g0, const int* off, const float* val, const bool* ok) {
#pragma unroll
    for (int i = 0; i < K; ++i)
      if (ok[i]) out[g0 + off[i]] = val[i];
  }
  __device__ __forceinline__ void finish() {}
};

// MVDeconvolution.computeQuotient (MVDeconvolution.java:494-546): img > 0 ? img / blurred : 1
struct EpiQuotient {
  const float* img;
  float* q;
  int nx, ny;
  int inputs(const float** p) const {
    p[0] = img;
    return 1;
  }
  __device__ __forceinline__ void acc_init() {}
  __device__ __forceinline__ static float quotient(float i, float blurred) {
    return i > 0.f ? __fdividef(i, blurred) : 1.f;  // within 2 ulp (blurred below 2^126)
  }
  __device__ __forceinline__ void operator()(long long g, float blurred) { q[g] = quotient(__ldg(img + g), blurred); }
  template <int K>
  __device__ __forceinline__ void apply(long long g0, const int* off, const float* val, const bool* ok) {
    constexpr int C = K < 8 ? K : 8;
#pragma unroll
    for (int c = 0; c < K; c += C) {
      float im[C];
#pragma unroll
      for (int i = 0; i < C; ++i) im[i] = (c + i < K && ok[c + i]) ? __ldg(img + g0 + off[c + i]) : 0.f;
#pragma unroll
      for (int i = 0; i < C; ++i)
        if (c + i < K && ok[c + i]) q[g0 + off[c + i]] = quotient(im[i], val[c + i]);
    }
  }
  __device__ __forceinline__ void finish() {}
};

// Where the update pass files a view's statistics once its last CTA is done: the history ring
// hist[(iteration % slots) * nviews + view] = (sum, max), after which the running sums are
// cleared for the view's next update and, after the last view, the iteration counter advances.
// `ticket` counts finished CTAs (the last one archives and resets it).  hist == nullptr: no
// archive (the sums are left for the caller).
struct StatArchive {
  double* hist;
  int* iter;
  unsigned* ticket;
  int view, nviews, slots;
};

// MVDeconvolution.computeFinalValues / computeNextValue / tikhonov (:603-726).  The reference
// evaluates tikhonov in double and rounds to float; here the algebraically equal form
// 2v / (sqrt(1 + 2 lambda v) + 1) is evaluated in float (no cancellation), its square root as
// x rsqrt(x) with x = 1 + 2 lambda v >= 1 and its division by the reciprocal intrinsic: within a
// few ulp.  At the overflow ends the result matches the IEEE form's: an infinite 2v stays
// infinite, and an infinite x gives NaN where the IEEE form gives 2v / inf = 0, both of which
// the clamp below turns into minValue.  Statistics (sum and max of |change|) are accumulated
// in FP64.
struct EpiUpdate {
  float* psi;
  const float* weight;
  float lambda;
  double* stat_sum;    // += sum |change| (FP64)
  unsigned* stat_max;  // max |change| as float bits (changes are >= 0)
  int nx, ny;
  float acc_sum;
  float acc_max;
  StatArchive archive;
  int inputs(const float** p) const {
    p[0] = psi;
    p[1] = weight;
    return 2;
  }
  __device__ __forceinline__ void acc_init() {
    acc_sum = 0.f;
    acc_max = 0.f;
  }
  __device__ __forceinline__ float next_value(float last, float integral, float w) {
    const float value = __fmul_rn(last, integral);
    float adjusted;
    if (value > 0.f) {
      if (lambda > 0.f && !isinf(value)) {
        const float x = __fadd_rn(1.f, __fmul_rn(2.f * lambda, value));
        const float r = __fmul_rn(x, rsqrtf(x));
        adjusted = __fdividef(__fmul_rn(2.f, value), __fadd_rn(r, 1.f));
      } else {
        adjusted = value;
      }
    } else {
      adjusted = 1e-4f;
    }
    const float next = isnan(adjusted) ? 1e-4f : fmaxf(1e-4f, adjusted);
    const float out = __fadd_rn(last, __fmul_rn(__fsub_rn(next, last), w));
    const float change = fabsf(__fsub_rn(out, last));
    acc_sum += change;
    acc_max = fmaxf(acc_max, change);
    return out;
  }
  __device__ __forceinline__ void operator()(long long g, float integral) {
    psi[g] = next_value(psi[g], integral, __ldg(weight + g));
  }
  template <int K>
  __device__ __forceinline__ void apply(long long g0, const int* off, const float* val, const bool* ok) {
    constexpr int C = K < 4 ? K : 4;
#pragma unroll
    for (int c = 0; c < K; c += C) {
      float last[C], w[C];
#pragma unroll
      for (int i = 0; i < C; ++i) {
        last[i] = (c + i < K && ok[c + i]) ? psi[g0 + off[c + i]] : 0.f;
        w[i] = (c + i < K && ok[c + i]) ? __ldg(weight + g0 + off[c + i]) : 0.f;
      }
#pragma unroll
      for (int i = 0; i < C; ++i)
        if (c + i < K && ok[c + i]) psi[g0 + off[c + i]] = next_value(last[i], val[c + i], w[i]);
    }
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
        if (archive.hist) {
          // the CTA that finishes last files the view's totals (the threadfence-reduction pattern:
          // every CTA's atomics are visible before its ticket)
          __threadfence();
          if (atomicAdd(archive.ticket, 1u) == gridDim.x - 1) {
            __threadfence();
            const double total = atomicAdd(stat_sum, 0.0);
            const unsigned mbits = atomicMax(stat_max, 0u);
            const int it = *archive.iter % archive.slots;
            archive.hist[(it * archive.nviews + archive.view) * 2 + 0] = total;
            archive.hist[(it * archive.nviews + archive.view) * 2 + 1] = (double)__uint_as_float(mbits);
            *stat_sum = 0.0;
            *stat_max = 0u;
            *archive.ticket = 0u;
            if (archive.view == archive.nviews - 1) *archive.iter += 1;
          }
        }
      }
    }
  }
};

// Poisson negative log-likelihood of the image-formation model and its residual:
// for img > 0: nll += w (f - img log f), r = w (1 - img / f); else r = 0.
// The per-thread partial sums are float; the CTA reduction and the global sum are FP64.
struct EpiNll {
  const float* img;
  const float* weight;
  float* r;           // residual out (may be null)
  double* nll;        // += sum over the CTA's voxels
  int nx, ny;
  float acc;
  int inputs(const float** p) const {
    p[0] = img;
    p[1] = weight;
    return 2;
  }
  __device__ __forceinline__ void acc_init() { acc = 0.f; }
  __device__ __forceinline__ float term(float f, float im, float w, float& res) {
    if (im > 0.f) {
      res = __fmul_rn(w, __fsub_rn(1.f, __fdiv_rn(im, f)));
      return w * (f - im * logf(f));
    }
    res = 0.f;
    return 0.f;
  }
  __device__ __forceinline__ void operator()(long long g, float f) {
    float res;
    acc += term(f, __ldg(img + g), __ldg(weight + g), res);
    if (r) r[g] = res;
  }
  template <int K>
  __device__ __forceinline__ void apply(long long g0, const int* off, const float* val, const bool* ok) {
    constexpr int C = K < 4 ? K : 4;
#pragma unroll
    for (int c = 0; c < K; c += C) {
      float im[C], w[C];
#pragma unroll
      for (int i = 0; i < C; ++i) {
        im[i] = (c + i < K && ok[c + i]) ? __ldg(img + g0 + off[c + i]) : 0.f;
        w[i] = (c + i < K && ok[c + i]) ? __ldg(weight + g0 + off[c + i]) : 0.f;
      }
#pragma unroll
      for (int i = 0; i < C; ++i) {
        if (c + i < K && ok[c + i]) {
          float res;
          acc += term(val[c + i], im[i], w[i], res);
          if (r) r[g0 + off[c + i]] = res;
        }
      }
    }
  }
  __device__ __forceinline__ void finish() {
    __shared__ double red[32];
    double sum = (double)acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = sum;
    __syncthreads();
    if (warp == 0) {
      sum = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
      if (lane == 0) atomicAdd(nll, sum);
    }
  }
};

// ------------------------------------------------------------------------------------------
// load / store functors of the first and last FFT stages
// ------------------------------------------------------------------------------------------
template <class Gather, bool MASK = false>
struct RowGather {  // packed pair (x[2n], x[2n+1]) of tile row `batch`, gathered from the volume
  Gather g;
  int ox, oy, gz;
  // MASK: values outside the tile's effective region [x0, x1) x [y0, y1) (slice inside: zin)
  int x0, x1, y0, y1;
  bool zin;
  template <int R>
  __device__ __forceinline__ void get(int batch, int j, int NR, float2* v) const {
    const auto row = g.row(oy + batch, gz);
    const bool yin = !MASK || (zin && batch >= y0 && batch < y1);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int lx = 2 * (j + r * NR);
      const int gx = ox + lx;
      float a = row(gx), b = row(gx + 1);
      if (MASK) {
        a = (yin && lx >= x0 && lx < x1) ? a : 0.f;
        b = (yin && lx + 1 >= x0 && lx + 1 < x1) ? b : 0.f;
      }
      v[r] = make_float2(a, b);
    }
  }
};

struct SpecSliceLoad {  // spectrum slice [y][kx]: batch = kx, i = y
  const float2* p;
  int px;
  template <int R>
  __device__ __forceinline__ void get(int batch, int j, int NR, float2* v) const {
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = __ldg(p + (j + r * NR) * px + batch);
  }
};

struct SpecSliceStore {
  float2* p;
  int px;
  template <int R>
  __device__ __forceinline__ void put(int batch, int base, int Ns, const float2* v) const {
#pragma unroll
    for (int r = 0; r < R; ++r) p[(base + r * Ns) * px + batch] = v[r];
  }
};

struct PencilRef {  // pencil element: batch = pencil in the chunk, i = z (32-bit offsets within a tile)
  float2* p;
  int plane;
  template <int R>
  __device__ __forceinline__ void get(int batch, int j, int NR, float2* v) const {
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = p[(j + r * NR) * plane + batch];
  }
  template <int R>
  __device__ __forceinline__ void put(int batch, int base, int Ns, const float2* v) const {
#pragma unroll
    for (int r = 0; r < R; ++r) p[(base + r * Ns) * plane + batch] = v[r];
  }
};

// Store of a convolution's last inverse z stage that keeps only the tile's effective slices
// [z0, z1): the inverse plane pass reads no other slice of the spectrum.
struct PencilEffectiveStore {
  float2* p;
  int plane, z0, z1;
  template <int R>
  __device__ __forceinline__ void put(int batch, int base, int Ns, const float2* v) const {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int z = base + r * Ns;
      if (z >= z0 && z < z1) p[z * plane + batch] = v[r];
    }
  }
};

struct PencilScaledStore {
  float2* p;
  int plane;
  float scale;
  template <int R>
  __device__ __forceinline__ void put(int batch, int base, int Ns, const float2* v) const {
#pragma unroll
    for (int r = 0; r < R; ++r) p[(base + r * Ns) * plane + batch] = cscale(v[r], scale);
  }
};

struct OtfMul {  // v[r] *= OTF at natural index j + r NR of pencil `batch`
  const float2* p;
  int plane;
  template <int R>
  __device__ __forceinline__ void apply(int batch, int j, int NR, float2* v) const {
    float2 o[R];
#pragma unroll
    for (int r = 0; r < R; ++r) o[r] = __ldg(p + (j + r * NR) * plane + batch);
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = cmul(v[r], o[r]);
  }
};

// First column stage of the forward plane pass: the half spectrum X[y][kx] of the real rows,
// formed on the fly from the packed row transforms Z (shared memory, rows of M complex):
// X[k] = e - i w^k o with e = (Z[k] + conj Z[M-k]) / 2, o = (Z[k] - conj Z[M-k]) / 2,
// X[0] = Re Z[0] + Im Z[0], X[M] = Re Z[0] - Im Z[0];  w = exp(-2 pi i / 2M).
struct R2CColumnLoad {
  const float2* z;
  int pitch, M;
  const float2* tw2;
  template <int R>
  __device__ __forceinline__ void get(int kx, int j, int NR, float2* v) const {
    if (kx == 0 || kx == M) {
      const float sg = kx == 0 ? 1.f : -1.f;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 z0 = z[(j + r * NR) * pitch];
        v[r] = make_float2(z0.x + sg * z0.y, 0.f);
      }
      return;
    }
    const float2 w = __ldg(tw2 + kx);
    const int kc = M - kx;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const float2* row = z + (j + r * NR) * pitch;
      const float2 zk = row[kx], zc = row[kc];
      const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y - zc.y));
      const float2 o = make_float2(0.5f * (zk.x - zc.x), 0.5f * (zk.y + zc.y));
      const float2 wo = cmul(w, o);
      v[r] = make_float2(e.x + wo.y, e.y - wo.x);
    }
  }
};

// First row stage of the inverse plane pass: the packed transform Z[k] of effective row
// `batch` formed from its half spectrum X (shared memory): Z[k] = (X[k] + conj X[M-k])
// + i conj(w^k) (X[k] - conj X[M-k]); with an unnormalised inverse FFT_M it yields 2M x.
struct C2RRowLoad {
  const float2* x;  // effective row 0
  int pitch, M;
  const float2* tw2;
  template <int R>
  __device__ __forceinline__ void get(int batch, int j, int NR, float2* v) const {
    const float2* row = x + batch * pitch;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int k = j + r * NR;
      const float2 xk = row[k], xc = row[k == 0 ? M : M - k];
      const float2 e = make_float2(xk.x + xc.x, xk.y - xc.y);
      const float2 o = make_float2(xk.x - xc.x, xk.y + xc.y);
      const float2 w = k == 0 ? make_float2(1.f, 0.f) : __ldg(tw2 + k);
      const float2 wo = cmul(cconj(w), o);
      v[r] = make_float2(e.x - wo.y, e.y + wo.x);
    }
  }
};

// All stages of one transform with the result left in shared memory: on return (after a
// barrier) `cur` holds it in the plain layout.  Stage 0 loads with ld0 (global memory or
// `cur`) and every stage writes the other buffer.  ROWS (row transforms, es == 1): stage 0
// (ROW_G0: it reads global memory) maps butterflies j-fastest for coalesced loads and writes
// the skewed layout; exchanges between shared buffers map them batch-fastest (one position of
// 32 consecutive rows per warp: conflict-free with an odd pitch).
template <bool INV, bool ROWS, bool ROW_G0, class LD0>
__device__ __forceinline__ void run_transform_smem(const FftPlan* __restrict__ p, int count, const LD0& ld0,
                                                   float2*& cur, float2*& oth, int es, int bs) {
  const int n = __ldg(&p->n);
  const int ns = __ldg(&p->nstages);
  const float2* tw = p->tw;
  int Ns = 1;
  for (int s = 0; s < ns; ++s) {
    const int R = __ldg(&p->radix[s]);
    const int skew_out = (ROWS && ROW_G0 && s == 0 && ns > 1) ? -1 : 0;
    const int skew_in = (ROWS && ROW_G0 && s == 1) ? -1 : 0;
    if (s == 0)
      stage<INV, ROWS && ROW_G0>(R, n, Ns, count, tw, ld0, Smem{oth, es, bs, skew_out});
    else
      stage<INV, false>(R, n, Ns, count, tw, Smem{cur, es, bs, skew_in}, Smem{oth, es, bs, 0});
    __syncthreads();
    float2* t = cur;
    cur = oth;
    oth = t;
    Ns *= R;
  }
}

// All stages of one transform with the last stage storing through `stl` (global memory or an
// epilogue).  Stage 0 loads with ld0; the exchanges in between alternate the two buffers.
// ROWS: the last stage (it writes global memory) maps butterflies j-fastest for coalesced
// stores, reading the skewed layout; earlier stages map them batch-fastest.
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
    if (s == ns - 1) {
      stage<INV, ROWS>(R, n, Ns, count, tw, Smem{cur, es, bs, ROWS ? -1 : 0}, stl);
    } else {
      const int skew_out = (ROWS && s == ns - 2) ? -1 : 0;
      if (s == 0)
        stage<INV, false>(R, n, Ns, count, tw, ld0, Smem{oth, es, bs, skew_out});
      else
        stage<INV, false>(R, n, Ns, count, tw, Smem{cur, es, bs, 0}, Smem{oth, es, bs, skew_out});
      __syncthreads();
      float2* t = cur;
      cur = oth;
      oth = t;
    }
    Ns *= R;
  }
}

// ------------------------------------------------------------------------------------------
// kernels (templated on gather / epilogue; instantiated in passes_*.cu)
// ------------------------------------------------------------------------------------------
// MASK: the gathered values are kept only inside the tile's effective region (tiles then
// partition the volume; used for the PSF gradient's correlation).
// src (count 0 or 1): tensor map of the gathered volume with a (tx rounded to 16 bytes + 4, ty,
// 1) box; each CTA prefetches into L2 the slice of the CTA `ahead` launches later.
template <class Gather, bool MASK = false>
__global__ void __launch_bounds__(kThreads, 2)
plane_fwd_kernel(const TileDesc* __restrict__ tiles, const int2* __restrict__ items,
                 const FftPlan* __restrict__ plans, float2* __restrict__ spec, Gather gather,
                 const __grid_constant__ EpiBoxes src, int ahead) {
  extern __shared__ float2 sm[];
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int z = it.y;
  if (threadIdx.x == 0 && src.count && blockIdx.x + ahead < gridDim.x) {
    const int2 it2 = items[blockIdx.x + ahead];
    const TileDesc t2 = tiles[it2.x];
    int zsrc;
    if (gather.slice_source(t2.oz + it2.y, zsrc)) prefetch_box_l2(&src.map[0], t2.ox & ~3, t2.oy, zsrc);
  }
  float cval;
  if (!MASK && gather.constant_slice(t.oz + z, cval)) {
    constant_spectrum_slice(spec + t.spec_off + (long long)z * t.ty * t.px, t.tx, t.ty, t.px, cval);
    return;
  }
  const int M = t.tx / 2;
  float2* cur = sm;
  float2* oth = sm + t.ty * t.pitch;
  // x: R2C of every row (packed pairs gathered straight from the volume)
  RowGather<Gather, MASK> ld0{gather, t.ox, t.oy, t.oz + z, t.hx, t.hx + t.ex, t.hy, t.hy + t.ey,
                              z >= t.hz && z < t.hz + t.ez};
  const FftPlan* pxp = plans + t.plan_x;
  run_transform_smem<false, true, true>(pxp, t.ty, ld0, cur, oth, 1, t.pitch);
  // y: C2C of every half-spectrum column (formed while loading), last stage straight to the
  // spectrum slice
  SpecSliceStore st{spec + t.spec_off + (long long)z * t.ty * t.px, t.px};
  run_transform_to<false, false>(plans + t.plan_y, t.px, R2CColumnLoad{cur, t.pitch, M, pxp->tw_r2c}, st, cur, oth,
                                 t.pitch, 1);
}

// boxes: tensor maps of the volumes the epilogue reads (count 0..2), prefetched into L2 for this
// slice's effective region at the start
template <class Epi>
__global__ void __launch_bounds__(kThreads, 2)
plane_inv_kernel(const TileDesc* __restrict__ tiles, const int2* __restrict__ items,
                 const FftPlan* __restrict__ plans, const float2* __restrict__ spec, Epi epi,
                 const __grid_constant__ EpiBoxes boxes) {
  extern __shared__ float2 sm[];
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int z = it.y;  // tile-local slice, inside the effective range
  if (threadIdx.x == 0)
    for (int i = 0; i < boxes.count; ++i) prefetch_box_l2(&boxes.map[i], (t.ox + t.hx) & ~3, t.oy + t.hy, t.oz + z);
  const int M = t.tx / 2;
  float2* cur = sm;
  float2* oth = sm + t.ty * t.pitch;
  // y: inverse C2C of every column, first stage straight from the spectrum slice
  SpecSliceLoad ld{spec + t.spec_off + (long long)z * t.ty * t.px, t.px};
  run_transform_smem<true, false, false>(plans + t.plan_y, t.px, ld, cur, oth, t.pitch, 1);
  // only the effective rows go on: the inverse x transform, its first stage forming the
  // packed transform of each row from the half spectrum while loading
  float2* rows = cur + t.hy * t.pitch;
  float2* rows_oth = oth + t.hy * t.pitch;
  const FftPlan* pxp = plans + t.plan_x;
  const long long gz = t.oz + z;
  // the C2R row transform stays in shared memory (batch-fastest stages), then the epilogue
  // walks the effective region by whole warps per row, so its global accesses coalesce
  run_transform_smem<true, true, false>(pxp, t.ey, C2RRowLoad{rows, t.pitch, M, pxp->tw_r2c}, rows, rows_oth, 1,
                                        t.pitch);
  const float* f = reinterpret_cast<const float*>(rows) + t.hx;
  const int lane = threadIdx.x & 31;
  epi.acc_init();
  for (int row = threadIdx.x >> 5; row < t.ey; row += blockDim.x >> 5) {
    const long long g0 = (gz * epi.ny + (t.oy + t.hy + row)) * (long long)epi.nx + t.ox + t.hx;
    const float* src = f + row * (2 * t.pitch);
    for (int x0 = 0; x0 < t.ex; x0 += 128) {
      int off[4];
      float val[4];
      bool ok[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int x = x0 + lane + 32 * u;
        off[u] = x;
        ok[u] = x < t.ex;
        val[u] = ok[u] ? src[x] : 0.f;
      }
      epi.template apply<4>(g0, off, val, ok);
    }
  }
  epi.finish();
}

// MODE 0: forward z, multiply by the OTF, inverse z (only the effective slices stored).
// MODE 1: forward z and scale (OTF build, spectra of the PSF gradient).  MODE 2: inverse z only.
// OCC: CTAs per SM the register allocation is sized for.
template <int MODE, int OCC = 2>
__global__ void __launch_bounds__(kZThreads, OCC)
zpass_kernel(const TileDesc* __restrict__ tiles, const int2* __restrict__ items,
             const FftPlan* __restrict__ plans, float2* __restrict__ spec,
             const float2* __restrict__ otf, float scale) {
  extern __shared__ float2 sm[];
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int p0 = it.y;
  const int plane = t.ty * t.px;
  const int count = min(kZChunk, plane - p0);
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
  if (MODE == 2) {  // inverse only
    run_transform_to<true, false>(pz, count, g, g, cur, oth, kZPitch, 1);
    return;
  }
  OtfMul mul{otf + t.otf_off + p0, plane};
  const PencilEffectiveStore ge{g.p, plane, t.hz, t.hz + t.ez};
  if (ns == 1) {
    zmid(__ldg(&pz->radix[0]), n, count, tw, g, mul, ge);
    return;
  }
  // forward stages 0 .. ns-2
  int Ns = 1;
  for (int s = 0; s < ns - 1; ++s) {
    const int R = __ldg(&pz->radix[s]);
    if (s == 0) {
      stage<false, false>(R, n, Ns, count, tw, g, Smem{cur, kZPitch, 1, 0});
    } else {
      stage<false, false>(R, n, Ns, count, tw, Smem{cur, kZPitch, 1, 0}, Smem{oth, kZPitch, 1, 0});
      float2* tmp = cur;
      cur = oth;
      oth = tmp;
    }
    __syncthreads();
    Ns *= R;
  }
  // forward last stage, product with the OTF, inverse first stage
  zmid(__ldg(&pz->radix[ns - 1]), n, count, tw, Smem{cur, kZPitch, 1, 0}, mul, Smem{oth, kZPitch, 1, 0});
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
      stage<true, false>(R, n, Ns, count, tw, Smem{cur, kZPitch, 1, 0}, ge);
    } else {
      stage<true, false>(R, n, Ns, count, tw, Smem{cur, kZPitch, 1, 0}, Smem{oth, kZPitch, 1, 0});
      __syncthreads();
      float2* tmp = cur;
      cur = oth;
      oth = tmp;
    }
    Ns *= R;
  }
}

}  // namespace mvd
