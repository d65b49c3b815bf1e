// Plane kernels with the tile shape fixed at compile time.
//
// The generic plane kernels (kernels.cuh) read the tile lengths, radices and strides from
// their plan at run time, so every stage carries index arithmetic on runtime values and the
// kernel carries every radix (a large body that misses the instruction cache).  For the tile
// shapes the planner picks most often, these kernels take (TX, TY, threads) as template
// parameters: the radix sequence, strides, butterfly counts and the twiddle stride are
// constants, divisions by them become multiplies, shared-memory offsets become immediates,
// and only the radices of the shape are compiled in.  The arithmetic (radix order, twiddles,
// functors, epilogues) is the generic kernels', so results are bit-identical to them.
#pragma once
#include "kernels.cuh"

namespace mvd {

// The planner's factorisation (engine.cu factorize): fewest stages, then the largest smallest
// radix, radices non-increasing, from {20, 18, 16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2}.
struct SplitC {
  int s = 0;
  int r[kMaxStages] = {0, 0, 0, 0, 0, 0};
};

constexpr int kRadixList[13] = {20, 18, 16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2};

__host__ __device__ constexpr int split_min(const SplitC& c) {
  int m = 1 << 30;
  for (int i = 0; i < c.s; ++i) m = c.r[i] < m ? c.r[i] : m;
  return c.s ? m : 0;
}

__host__ __device__ constexpr void split_search(int n, int depth, int maxdepth, SplitC& cur, SplitC& best, bool& found) {
  if (n == 1) {
    if (!found || cur.s < best.s || (cur.s == best.s && split_min(cur) > split_min(best))) {
      best = cur;
      found = true;
    }
    return;
  }
  if (depth == maxdepth) return;
  for (int i = 0; i < 13; ++i) {
    const int r = kRadixList[i];
    if (n % r) continue;
    if (cur.s && r > cur.r[cur.s - 1]) continue;
    cur.r[cur.s++] = r;
    split_search(n / r, depth + 1, maxdepth, cur, best, found);
    --cur.s;
  }
}

__host__ __device__ constexpr SplitC split_of(int n) {
  SplitC cur{}, best{};
  bool found = false;
  if (n == 1) {
    best.s = 1;
    best.r[0] = 1;
    return best;
  }
  for (int d = 1; d <= kMaxStages && !found; ++d) split_search(n, 0, d, cur, best, found);
  return best;
}

// Voxels per lane of one step of the inverse passes' epilogue walk (a warp per effective row):
// enough for a whole row of a TX-wide tile, so that a row of, say, 130 voxels takes one step
// instead of a 128-voxel step and a 2-voxel one.
template <int TX>
constexpr int kEpiPerLane = (TX + 31) / 32;

// Shared-memory accessor with compile-time strides: element (batch, i) at
// p[batch * BS + s(i) * ES], s(i) = i or the skewed i + i/16.
template <int ES, int BS, bool SKEW>
struct SmemC {
  float2* p;
  __device__ __forceinline__ static int at(int batch, int i) { return batch * BS + (SKEW ? i + (i >> 4) : i) * ES; }
  template <int R>
  __device__ __forceinline__ void get(int batch, int j, int NR, float2* v) const {
    if (SKEW) {
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = p[at(batch, j + r * NR)];
    } else {
      const float2* q = p + batch * BS + j * ES;
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = q[r * NR * ES];
    }
  }
  template <int R>
  __device__ __forceinline__ void put(int batch, int base, int Ns, const float2* v) const {
    if (SKEW) {
#pragma unroll
      for (int r = 0; r < R; ++r) p[at(batch, base + r * Ns)] = v[r];
    } else {
      float2* q = p + batch * BS + base * ES;
#pragma unroll
      for (int r = 0; r < R; ++r) q[r * Ns * ES] = v[r];
    }
  }
};

// One radix-R Stockham stage over `count` sequences of length N (Ns = product of the earlier
// radices), T threads; the generic stage_r with N, Ns, R and T constant.
template <int R, int N, int NS, bool INV, bool JFAST, int T, class LD, class ST>
__device__ __forceinline__ void stage_c(int count, const float2* __restrict__ tw, const LD& ld, const ST& st) {
  constexpr int NR = N / R;
  constexpr int TWS = N / (NS * R);
  const int nb = count * NR;
  const int fast = JFAST ? NR : count;
  for (int b = threadIdx.x; b < nb; b += T) {
    const int sl = b / fast;
    const int f = b - sl * fast;
    const int batch = JFAST ? sl : f;
    const int j = JFAST ? f : sl;
    float2 v[R];
    ld.template get<R>(batch, j, NR, v);
    const int k = NS > 1 ? j % NS : 0;
    if (NS > 1 && k != 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 w = __ldg(tw + r * k * TWS);
        if (INV) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    Dft<R, INV>::run(v);
    st.template put<R>(batch, (j - k) * R + k, NS, v);
  }
}

template <int N>
__host__ __device__ constexpr int ns_before(int s) {
  int p = 1;
  for (int i = 0; i < s; ++i) p *= split_of(N).r[i];
  return p;
}

// Stages s .. S-1 of a length-N transform whose result stays in shared memory (the generic
// run_transform_smem): stage 0 loads with ld0, every stage writes the other buffer.
// SKEW: the first row stage (ROW_G0) writes the skewed layout i + i/16 and the second reads it.
template <int N, int s, bool INV, bool ROWS, bool ROW_G0, int ES, int BS, int T, bool SKEW = true, class LD0>
__device__ __forceinline__ void smem_stages(int count, const float2* __restrict__ tw, const LD0& ld0, float2*& cur,
                                            float2*& oth) {
  constexpr SplitC sp = split_of(N);
  if constexpr (s < sp.s) {
    constexpr int R = sp.r[s];
    constexpr int NS = ns_before<N>(s);
    if constexpr (s == 0) {
      constexpr bool skew_out = SKEW && ROWS && ROW_G0 && sp.s > 1;
      stage_c<R, N, NS, INV, ROWS && ROW_G0, T>(count, tw, ld0, SmemC<ES, BS, skew_out>{oth});
    } else {
      constexpr bool skew_in = SKEW && ROWS && ROW_G0 && s == 1;
      stage_c<R, N, NS, INV, false, T>(count, tw, SmemC<ES, BS, skew_in>{cur}, SmemC<ES, BS, false>{oth});
    }
    __syncthreads();
    float2* t = cur;
    cur = oth;
    oth = t;
    smem_stages<N, s + 1, INV, ROWS, ROW_G0, ES, BS, T, SKEW>(count, tw, ld0, cur, oth);
  }
}

// Shared-memory row layout of a compiled plane shape, chosen per shape with a wavefront model of
// the forward pass's shared accesses (float2 accesses, 16 bank pairs per half warp): whether the
// first row stage, which maps butterflies j-fastest, writes the skewed layout i + i/16, and the
// row pitch (odd, so that batch-fastest row stages are conflict-free).  The skew suits 128-wide
// tiles (radix 8 x 8); for 100, 160 and 192-wide tiles the plain layout gives 7-46% fewer
// wavefronts (160x160: 4986 against 9280 per slice), because their first-stage stride (10 or
// 12) already spreads a row's positions over the banks.
__host__ __device__ constexpr bool fixed_skew(int TX) { return TX == 128; }
__host__ __device__ constexpr int fixed_pitch(int TX) { return fixed_skew(TX) ? row_pitch(TX / 2) : ((TX / 2 + 1) | 1); }

// All stages with the last storing through stl (the generic run_transform_to).
template <int N, int s, bool INV, bool ROWS, int ES, int BS, int T, class LD0, class STL>
__device__ __forceinline__ void to_stages(int count, const float2* __restrict__ tw, const LD0& ld0, const STL& stl,
                                          float2*& cur, float2*& oth) {
  constexpr SplitC sp = split_of(N);
  constexpr int R = sp.r[s];
  constexpr int NS = ns_before<N>(s);
  if constexpr (sp.s == 1) {
    stage_c<R, N, 1, INV, ROWS, T>(count, tw, ld0, stl);
  } else if constexpr (s == sp.s - 1) {
    stage_c<R, N, NS, INV, ROWS, T>(count, tw, SmemC<ES, BS, ROWS>{cur}, stl);
  } else {
    constexpr bool skew_out = ROWS && s == sp.s - 2;
    if constexpr (s == 0)
      stage_c<R, N, NS, INV, false, T>(count, tw, ld0, SmemC<ES, BS, skew_out>{oth});
    else
      stage_c<R, N, NS, INV, false, T>(count, tw, SmemC<ES, BS, false>{cur}, SmemC<ES, BS, skew_out>{oth});
    __syncthreads();
    float2* t = cur;
    cur = oth;
    oth = t;
    to_stages<N, s + 1, INV, ROWS, ES, BS, T>(count, tw, ld0, stl, cur, oth);
  }
}

// CTAs per SM a compiled-shape plane kernel is sized for: two when two CTAs' buffers (two
// planes of TY rows at the row pitch each) fit the SM's shared memory, else one.  The register
// allocation follows (T threads x CTAs within the 64K registers of an SM).  Planes of up to
// ~100 KB per buffer run 512-thread CTAs, two per SM; larger planes run one 1024-thread CTA per
// SM, so that twice as many warps hide the latency of the gathers and the exchanges (on the
// 512x512x256 workload 1024 threads measured 23.5 G voxel-updates/s, 768 threads 23.0, 512
// threads 21.3).  The in-place kernels of those shapes (fixed_plane_tm.cuh) keep one buffer and
// run two 512-thread CTAs per SM instead.
__host__ __device__ constexpr int fixed_ctas_per_sm(int TX, int TY) {
  return 2 * (2 * TY * row_pitch(TX / 2) * 8) <= 227 * 1024 ? 2 : 1;
}

// Forward plane pass: the generic kernel's structure (the first row stage gathers straight from
// the volume, j-fastest) with the shape fixed.  Staging the slice in shared memory first, for
// coalesced warp-per-row loads, measured slower on cfg2 (0.69 vs 0.64 ms per iteration): the
// j-fastest gather mostly hits L1 and saves a shared-memory pass and a barrier.
// `src` (count 0 or 1): tensor map of the gathered volume with a (TX rounded to 16 bytes + 4,
// TY, 1) box; each CTA prefetches into L2 the slice of the CTA `ahead` launches later (one
// resident wave on), so the next wave's gathers find their rows there.
template <class Gather, int TX, int TY, int T>
__global__ void __launch_bounds__(T, fixed_ctas_per_sm(TX, TY))
plane_fwd_fixed(const TileDesc* __restrict__ tiles, const int2* __restrict__ items, const FftPlan* __restrict__ plans,
                float2* __restrict__ spec, Gather gather, const __grid_constant__ EpiBoxes src, int ahead) {
  constexpr int M = TX / 2, PX = M + 1, PITCH = fixed_pitch(TX);
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
  if (gather.constant_slice(t.oz + z, cval)) {  // a slice of the extension value only
    constant_spectrum_slice(spec + t.spec_off + (long long)z * TY * PX, TX, TY, PX, cval);
    return;
  }
  float2* cur = sm;
  float2* oth = sm + TY * PITCH;
  RowGather<Gather, false> ld0{gather, t.ox, t.oy, t.oz + z, 0, 0, 0, 0, true};
  const FftPlan* pxp = plans + t.plan_x;
  smem_stages<M, 0, false, true, true, 1, PITCH, T, fixed_skew(TX)>(TY, pxp->tw, ld0, cur, oth);
  SpecSliceStore st{spec + t.spec_off + (long long)z * TY * PX, PX};
  to_stages<TY, 0, false, false, PITCH, 1, T>(PX, plans[t.plan_y].tw, R2CColumnLoad{cur, PITCH, M, pxp->tw_r2c}, st,
                                             cur, oth);
}

// Inverse plane pass.  The column stages are the generic kernel's; the C2R row transform of the
// effective rows stays in shared memory (batch-fastest stages), and the epilogue then walks the
// effective region by whole warps per row: psi / weight / img accesses are fully coalesced.
template <class Epi, int TX, int TY, int T>
__global__ void __launch_bounds__(T, fixed_ctas_per_sm(TX, TY))
plane_inv_fixed(const TileDesc* __restrict__ tiles, const int2* __restrict__ items, const FftPlan* __restrict__ plans,
                const float2* __restrict__ spec, Epi epi, const __grid_constant__ EpiBoxes boxes) {
  constexpr int M = TX / 2, PX = M + 1, PITCH = fixed_pitch(TX);
  extern __shared__ float2 sm[];
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int z = it.y;
  // this slice's epilogue inputs (prefetching the next resident wave's as well measured slower:
  // 27.29 vs 27.57 G voxel-updates/s on cfg2)
  if (threadIdx.x == 0)
    for (int i = 0; i < boxes.count; ++i) prefetch_box_l2(&boxes.map[i], (t.ox + t.hx) & ~3, t.oy + t.hy, t.oz + z);
  float2* cur = sm;
  float2* oth = sm + TY * PITCH;
  SpecSliceLoad ld{spec + t.spec_off + (long long)z * TY * PX, PX};
  smem_stages<TY, 0, true, false, false, PITCH, 1, T>(PX, plans[t.plan_y].tw, ld, cur, oth);
  float2* rows = cur + t.hy * PITCH;
  float2* rows_oth = oth + t.hy * PITCH;
  const FftPlan* pxp = plans + t.plan_x;
  smem_stages<M, 0, true, true, false, 1, PITCH, T>(t.ey, pxp->tw, C2RRowLoad{rows, PITCH, M, pxp->tw_r2c}, rows,
                                                    rows_oth);
  // rows: the real rows (x = 2n + c of packed element n), tile-local x from 0
  const float* f = reinterpret_cast<const float*>(rows) + t.hx;
  const long long gz = t.oz + z;
  const int lane = threadIdx.x & 31;
  epi.acc_init();
  for (int row = threadIdx.x >> 5; row < t.ey; row += T / 32) {
    const long long g0 = (gz * epi.ny + (t.oy + t.hy + row)) * (long long)epi.nx + t.ox + t.hx;
    const float* src = f + row * (2 * PITCH);
    constexpr int U = kEpiPerLane<TX>;  // one step covers any effective row (ex <= TX)
    for (int x0 = 0; x0 < t.ex; x0 += 32 * U) {
      int off[U];
      float val[U];
      bool ok[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int x = x0 + lane + 32 * u;
        off[u] = x;
        ok[u] = x < t.ex;
        val[u] = ok[u] ? src[x] : 0.f;
      }
      epi.template apply<U>(g0, off, val, ok);
    }
  }
  epi.finish();
}

// Forward last stage + product with the OTF + inverse first stage in registers (the generic
// zmid_r) for a length-N pencil with radix R = the last forward radix.
template <int R, int N, int T, class LD, class MUL, class ST>
__device__ __forceinline__ void zmid_c(int count, const float2* __restrict__ tw, const LD& ld, const MUL& mul,
                                       const ST& st) {
  constexpr int NR = N / R;
  const int nb = count * NR;
  for (int b = threadIdx.x; b < nb; b += T) {
    const int j = b / count;
    const int batch = b - j * count;
    float2 v[R];
    ld.template get<R>(batch, j, NR, v);
    if (j != 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(tw + r * j));
    }
    Dft<R, false>::run(v);
    mul.template apply<R>(batch, j, NR, v);
    Dft<R, true>::run(v);
    st.template put<R>(batch, j * R, 1, v);
  }
}

// Forward stages 1 .. S-2 of the z pencils (stage 0 is done by the caller), shared to shared.
template <int N, int s, int T>
__device__ __forceinline__ void z_fwd_stages(int count, const float2* __restrict__ tw, float2*& cur, float2*& oth) {
  constexpr SplitC sp = split_of(N);
  if constexpr (s < sp.s - 1) {
    stage_c<sp.r[s], N, ns_before<N>(s), false, false, T>(count, tw, SmemC<kZPitch, 1, false>{cur},
                                                          SmemC<kZPitch, 1, false>{oth});
    float2* t = cur;
    cur = oth;
    oth = t;
    __syncthreads();
    z_fwd_stages<N, s + 1, T>(count, tw, cur, oth);
  }
}

// Inverse stages i = 1 .. S-1 (radices in reverse order); the last stores through g.
template <int N, int i, int T, class G>
__device__ __forceinline__ void z_inv_stages(int count, const float2* __restrict__ tw, const G& g, float2*& cur,
                                             float2*& oth) {
  constexpr SplitC sp = split_of(N);
  if constexpr (i < sp.s) {
    constexpr int R = sp.r[sp.s - 1 - i];
    // Ns = the product of the radices already inverted: r[S-1] ... r[S-i]
    constexpr int NS = N / ns_before<N>(sp.s - i);
    if constexpr (i == sp.s - 1) {
      stage_c<R, N, NS, true, false, T>(count, tw, SmemC<kZPitch, 1, false>{cur}, g);
    } else {
      stage_c<R, N, NS, true, false, T>(count, tw, SmemC<kZPitch, 1, false>{cur}, SmemC<kZPitch, 1, false>{oth});
      __syncthreads();
      float2* t = cur;
      cur = oth;
      oth = t;
      z_inv_stages<N, i + 1, T>(count, tw, g, cur, oth);
    }
  }
}

// The z pass of a convolution (forward z, times the OTF, inverse z: the generic zpass_kernel
// in MODE 0) with the pencil length TZ fixed at compile time.
template <int TZ, int OCC>
__global__ void __launch_bounds__(kZThreads, OCC)
zpass_fixed(const TileDesc* __restrict__ tiles, const int2* __restrict__ items, const FftPlan* __restrict__ plans,
            float2* __restrict__ spec, const float2* __restrict__ otf) {
  constexpr SplitC sp = split_of(TZ);
  extern __shared__ float2 sm[];
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int p0 = it.y;
  const int plane = t.ty * t.px;
  const int count = min(kZChunk, plane - p0);
  const float2* tw = plans[t.plan_z].tw;
  float2* cur = sm;
  float2* oth = sm + TZ * kZPitch;
  PencilRef g{spec + t.spec_off + p0, plane};
  OtfMul mul{otf + t.otf_off + p0, plane};
  const PencilEffectiveStore ge{g.p, plane, t.hz, t.hz + t.ez};  // the inverse pass's slices only
  if constexpr (sp.s == 1) {
    zmid_c<sp.r[0], TZ, kZThreads>(count, tw, g, mul, ge);
  } else {
    // forward stage 0 straight from the pencils into `cur`, then the shared stages
    stage_c<sp.r[0], TZ, 1, false, false, kZThreads>(count, tw, g, SmemC<kZPitch, 1, false>{cur});
    __syncthreads();
    z_fwd_stages<TZ, 1, kZThreads>(count, tw, cur, oth);
    zmid_c<sp.r[sp.s - 1], TZ, kZThreads>(count, tw, SmemC<kZPitch, 1, false>{cur}, mul, SmemC<kZPitch, 1, false>{oth});
    __syncthreads();
    float2* tmp = cur;
    cur = oth;
    oth = tmp;
    z_inv_stages<TZ, 1, kZThreads>(count, tw, ge, cur, oth);
  }
}

// CTAs per SM a compiled z pass of length TZ is sized for: three when their shared memory (two
// buffers of TZ x kZPitch complex each) fits, else two (with the registers two allow).
__host__ __device__ constexpr int zpass_fixed_occ(int TZ) {
  return 3 * 2 * TZ * kZPitch * 8 <= 227 * 1024 ? 3 : 2;
}

// Loader of the inverse stage after the in-place middle stage of zpass_ip: butterfly j reads the
// R consecutive elements j R ... j R + R - 1 of its pencil (rows of PITCH complex).
template <int PITCH>
struct ZRowsLoad {
  const float2* p;
  template <int R>
  __device__ __forceinline__ void get(int batch, int j, int, float2* v) const {
    const float2* q = p + batch + j * R * PITCH;
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = q[r * PITCH];
  }
};

// zpass_fixed for two-stage pencil lengths TZ = R0 x R1 with ONE shared buffer, CH pencils per
// CTA of T threads.  The middle stage (forward radix R1, product with the OTF, inverse radix
// R1) writes each butterfly's results back to the positions it read them from (j + r R0),
// instead of the Stockham order (j R1 + r): no other thread touches those positions, so the
// stage needs neither a second buffer nor a barrier between its loads and stores.  Element
// e = a R1 + c of the Stockham order then sits at a + c R0, so the inverse radix-R0 stage, whose
// butterfly j wants elements j + r R1 (a = r, c = j), reads positions j R0 + r (ZRowsLoad).
// Arithmetic, twiddles and the order of operations are zpass_fixed's, so the effective slices
// are bit-identical to its output; the halo slices (outside [hz, hz + ez)), which the inverse
// plane pass never reads, are not stored.
//
// The host runs it with 32 pencils per CTA (kZWideChunk), 256 or 320 threads (zpass_ip_threads)
// and two CTAs per SM:
// the one buffer (TZ x 33 complex, 84 KB for 320) takes what two 16-pencil buffers took, and
// each z slice of a chunk is one 256-byte row in HBM instead of 128 bytes.  On the 512x512x256
// workload the z pass took 2.79 ms per iteration against 3.36 ms for the two-buffer kernel.  16
// pencils with four CTAs per SM (64 registers) took 3.80 ms, 32 pencils with 512 threads 3.83,
// 64 pencils with 512 threads and one CTA 3.16.
template <int TZ, int CH, int T, int OCC>
__global__ void __launch_bounds__(T, OCC)
zpass_ip(const TileDesc* __restrict__ tiles, const int2* __restrict__ items, const FftPlan* __restrict__ plans,
         float2* __restrict__ spec, const float2* __restrict__ otf) {
  constexpr SplitC sp = split_of(TZ);
  static_assert(sp.s == 2, "the in-place z pass is written for two-stage pencil lengths");
  constexpr int R0 = sp.r[0];
  constexpr int R1 = sp.r[1];
  constexpr int PITCH = CH + 1;
  extern __shared__ float2 sm[];
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int p0 = it.y;
  const int plane = t.ty * t.px;
  const int count = min(CH, plane - p0);
  const float2* tw = plans[t.plan_z].tw;
  const SmemC<PITCH, 1, false> buf{sm};
  PencilRef g{spec + t.spec_off + p0, plane};
  OtfMul mul{otf + t.otf_off + p0, plane};
  // forward stage 0 straight from the pencils: butterfly j's outputs at j R0 + r
  stage_c<R0, TZ, 1, false, false, T>(count, tw, g, buf);
  __syncthreads();
  {
    const int nb = count * R0;  // R0 butterflies of radix R1 per pencil
    for (int b = threadIdx.x; b < nb; b += T) {
      const int j = b / count;
      const int batch = b - j * count;
      float2 v[R1];
      buf.template get<R1>(batch, j, R0, v);
      if (j != 0) {
#pragma unroll
        for (int r = 1; r < R1; ++r) v[r] = cmul(v[r], __ldg(tw + r * j));
      }
      Dft<R1, false>::run(v);
      mul.template apply<R1>(batch, j, R0, v);
      Dft<R1, true>::run(v);
      buf.template put<R1>(batch, j, R0, v);
    }
  }
  __syncthreads();
  // the inverse plane pass reads the effective slices only: the halo slices are not stored
  stage_c<R0, TZ, R1, true, false, T>(count, tw, ZRowsLoad<PITCH>{sm},
                                      PencilEffectiveStore{g.p, plane, t.hz, t.hz + t.ez});
}

// CTA size of the in-place z pass: 320 threads for the 320 / 288 pencils (their middle stage's
// 640 / 576 butterflies of a 32-pencil chunk take two rounds instead of three; z pass 2.68 vs
// 2.72 ms per iteration on the 512x512x256 workload, 384 threads 2.89), else 256.
__host__ __device__ constexpr int zpass_ip_threads(int TZ) { return (TZ == 320 || TZ == 288) ? 320 : kZThreads; }

// Pencil lengths with compiled z-pass kernels: the 4-view 256x256x192 workload's (240, 216)
// and the 512x512x256 workload's (320, 288).
#define MVD_FIXED_Z_LENGTHS(X) \
  X(240)                       \
  X(216)                       \
  X(320)                       \
  X(288)

// Tile shapes (x length, y length, CTA size) with compiled kernels.  They replace the default
// 384-thread generic kernels: a plan whose CTA size is the default runs them at their own size.
// 100x100 and 128x100: the 256x256x192 workload's planes (two CTAs per SM); 160x160, 192x96 and
// 192x135: the 512x512x256 workload's (one 1024-thread CTA per SM with two buffers; by default
// these shapes run the in-place kernels of fixed_plane_tm.cuh, two 512-thread CTAs per SM).
#define MVD_FIXED_PLANE_SHAPES(X) \
  X(100, 100, 512)                \
  X(128, 100, 512)                \
  X(160, 160, 1024)               \
  X(192, 96, 1024)                \
  X(192, 135, 1024)

}  // namespace mvd
