// Plane kernels with one shared-memory buffer: every exchange stage runs in place, staged
// through the thread's own tensor-memory columns.
//
// The compile-time-shaped plane kernels (fixed_plane.cuh) ping-pong between two plane buffers.
// For the large planes (160x160, 192x96, 192x135: 75-105 KB per buffer) the two buffers leave
// room for one CTA per SM, which then runs 1024 threads, and every barrier of a slice stalls the
// whole SM.  On shapes that fit either way, two 512-thread CTAs per SM measured 16% faster on the
// plane passes than one 1024-thread CTA (1.35 against 1.57 ms per iteration on the 256x256x192
// workload), because one CTA's barrier waits overlap the other's work.
//
// Here a stage whose input and output are both the plane buffer runs in two phases: each thread
// loads, twiddles and transforms its butterflies (all rounds) and parks the results in its own
// tensor-memory columns (tcgen05.st), then -- after a barrier -- reads them back (tcgen05.ld) and
// writes them to their output positions.  Tensor memory can only be reached from the thread's own
// lane, which is why it serves as per-thread staging and not as a second exchange buffer.  Each
// CTA allocates 256 of the SM's 512 columns; its 16 warps take 64 columns per thread (warp w:
// lane quadrant w % 4, columns 64 (w / 4) ...), which holds every stage's rounds of these shapes.
// Stages that read or write global memory (the gather, the spectrum stores and loads) need no
// staging.  The arithmetic, loads and stores are those of the two-buffer kernels, so results are
// bit-identical to them.  No wait in these kernels depends on another CTA or on an asynchronous
// copy: the tensor-memory loads and stores complete under tcgen05.wait, and the allocation waits
// only for columns the SM's other CTA frees when it ends.
#pragma once
#include "fixed_plane.cuh"
#include "tcgen05.cuh"

namespace mvd {

constexpr int kTmThreads = 512;  // two CTAs per SM
constexpr int kTmCols = 256;     // tensor-memory columns per CTA (half of an SM's)
constexpr int kTmThreadCols = 64;

namespace tc {

#define MVD_TM_REGS16(v)                                                                                  \
  "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),                   \
      "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),               \
      "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),               \
      "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),             \
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),            \
      "r"(__float_as_uint(v[15]))

__device__ __forceinline__ void st_x16(uint32_t a, const float* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16};" ::"r"(a),
      MVD_TM_REGS16(v)
      : "memory");
}
__device__ __forceinline__ void st_x8(uint32_t a, const float* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(a),
               "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
               "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
               "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
               : "memory");
}
__device__ __forceinline__ void st_x4(uint32_t a, const float* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(__float_as_uint(v[0])),
               "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3]))
               : "memory");
}
__device__ __forceinline__ void st_x2(uint32_t a, const float* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1, %2};" ::"r"(a), "r"(__float_as_uint(v[0])),
               "r"(__float_as_uint(v[1]))
               : "memory");
}
#undef MVD_TM_REGS16

__device__ __forceinline__ void ld_x16(uint32_t a, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(a));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void ld_x8(uint32_t a, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(a));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void ld_x4(uint32_t a, float* v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void ld_x2(uint32_t a, float* v) {
  uint32_t r[2];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(a));
  v[0] = __uint_as_float(r[0]);
  v[1] = __uint_as_float(r[1]);
}

// NC consecutive columns (NC even) from / to registers, in chunks of 16, 8, 4 and 2 columns.
template <int NC>
__device__ __forceinline__ void tmem_store(uint32_t a, const float* v) {
  if constexpr (NC >= 16) {
    st_x16(a, v);
    tmem_store<NC - 16>(a + 16, v + 16);
  } else if constexpr (NC >= 8) {
    st_x8(a, v);
    tmem_store<NC - 8>(a + 8, v + 8);
  } else if constexpr (NC >= 4) {
    st_x4(a, v);
    tmem_store<NC - 4>(a + 4, v + 4);
  } else if constexpr (NC >= 2) {
    st_x2(a, v);
    tmem_store<NC - 2>(a + 2, v + 2);
  }
}
template <int NC>
__device__ __forceinline__ void tmem_load(uint32_t a, float* v) {
  if constexpr (NC >= 16) {
    ld_x16(a, v);
    tmem_load<NC - 16>(a + 16, v + 16);
  } else if constexpr (NC >= 8) {
    ld_x8(a, v);
    tmem_load<NC - 8>(a + 8, v + 8);
  } else if constexpr (NC >= 4) {
    ld_x4(a, v);
    tmem_load<NC - 4>(a + 4, v + 4);
  } else if constexpr (NC >= 2) {
    ld_x2(a, v);
    tmem_load<NC - 2>(a + 2, v + 2);
  }
}

}  // namespace tc

// One radix-R Stockham stage of `count` sequences (batch-fastest), in place: phase 1 loads,
// twiddles and transforms all of this thread's butterflies (ROUNDS of them at most) into its
// tensor-memory columns from `tcol`, phase 2 stores them.  The arithmetic is stage_c's.
template <int R, int N, int NS, bool INV, int T, int ROUNDS, class LD, class ST>
__device__ __forceinline__ void stage_staged(int count, const float2* __restrict__ tw, const LD& ld, const ST& st,
                                             uint32_t tcol) {
  static_assert(ROUNDS * 2 * R <= kTmThreadCols, "a stage's rounds must fit the thread's tensor-memory columns");
  constexpr int NR = N / R;
  constexpr int TWS = N / (NS * R);
  const int nb = count * NR;
#pragma unroll 1
  for (int k = 0; k < ROUNDS; ++k) {
    const int b = threadIdx.x + k * T;
    float2 v[R];
    if (b < nb) {
      const int j = b / count;
      const int batch = b - j * count;
      ld.template get<R>(batch, j, NR, v);
      const int kk = NS > 1 ? j % NS : 0;
      if (NS > 1 && kk != 0) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          float2 w = __ldg(tw + r * kk * TWS);
          if (INV) w.y = -w.y;
          v[r] = cmul(v[r], w);
        }
      }
      Dft<R, INV>::run(v);
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = make_float2(0.f, 0.f);
    }
    tc::tmem_store<2 * R>(tcol + k * 2 * R, reinterpret_cast<const float*>(v));  // the whole warp stores
  }
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
#pragma unroll 1
  for (int k = 0; k < ROUNDS; ++k) {
    const int b = threadIdx.x + k * T;
    float2 v[R];
    tc::tmem_load<2 * R>(tcol + k * 2 * R, reinterpret_cast<float*>(v));  // the whole warp loads
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (b < nb) {
      const int j = b / count;
      const int batch = b - j * count;
      const int kk = NS > 1 ? j % NS : 0;
      st.template put<R>(batch, (j - kk) * R + kk, NS, v);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
}

__host__ __device__ constexpr int ceil_div(int a, int b) { return (a + b - 1) / b; }

// The largest number of effective rows the inverse pass's row stages stage within the thread's
// columns for a TX-wide tile (the host runs these kernels only for plans within it).
template <int TX, int TY>
__host__ __device__ constexpr int tm_max_rows() {
  constexpr SplitC sx = split_of(TX / 2);
  int ey = TY;
  while (ey > 0 && (ceil_div(ey * (TX / 2 / sx.r[0]), kTmThreads) * 2 * sx.r[0] > kTmThreadCols ||
                    ceil_div(ey * (TX / 2 / sx.r[1]), kTmThreads) * 2 * sx.r[1] > kTmThreadCols))
    --ey;
  return ey;
}

// this thread's first tensor-memory column (lane quadrant warp % 4, column block warp / 4)
__device__ __forceinline__ uint32_t tm_thread_col(uint32_t base) {
  const int warp = threadIdx.x >> 5;
  return base + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(kTmThreadCols * (warp >> 2));
}

template <class Gather, int TX, int TY>
__global__ void __launch_bounds__(kTmThreads, 2)
plane_fwd_tm(const TileDesc* __restrict__ tiles, const int2* __restrict__ items, const FftPlan* __restrict__ plans,
             float2* __restrict__ spec, Gather gather, const __grid_constant__ EpiBoxes src, int ahead) {
  constexpr int M = TX / 2, PX = M + 1, PITCH = fixed_pitch(TX), T = kTmThreads;
  constexpr SplitC sx = split_of(M), sy = split_of(TY);
  static_assert(sx.s == 2 && sy.s == 2 && !fixed_skew(TX), "two-stage lengths in the plain row layout");
  extern __shared__ float2 sm[];
  __shared__ uint32_t tslot;
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
  if (threadIdx.x < 32) tc::tmem_alloc(&tslot, kTmCols);
  float2* a = sm;
  const FftPlan* pxp = plans + t.plan_x;
  const float2* twx = pxp->tw;
  const float2* twy = plans[t.plan_y].tw;
  // x stage 0 straight from the volume (j-fastest) into the buffer
  RowGather<Gather, false> ld0{gather, t.ox, t.oy, t.oz + z, 0, 0, 0, 0, true};
  stage_c<sx.r[0], M, 1, false, true, T>(TY, twx, ld0, SmemC<1, PITCH, false>{a});
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tcol = tm_thread_col(tslot);
  // x stage 1 and y stage 0 (the real-to-half-spectrum step folded into its loads) in place
  stage_staged<sx.r[1], M, sx.r[0], false, T, ceil_div(TY * (M / sx.r[1]), T)>(
      TY, twx, SmemC<1, PITCH, false>{a}, SmemC<1, PITCH, false>{a}, tcol);
  stage_staged<sy.r[0], TY, 1, false, T, ceil_div(PX * (TY / sy.r[0]), T)>(
      PX, twy, R2CColumnLoad{a, PITCH, M, pxp->tw_r2c}, SmemC<PITCH, 1, false>{a}, tcol);
  if (threadIdx.x < 32) tc::tmem_dealloc(tslot, kTmCols);
  // y stage 1 straight to the spectrum slice
  SpecSliceStore st{spec + t.spec_off + (long long)z * TY * PX, PX};
  stage_c<sy.r[1], TY, sy.r[0], false, false, T>(PX, twy, SmemC<PITCH, 1, false>{a}, st);
}

template <class Epi, int TX, int TY>
__global__ void __launch_bounds__(kTmThreads, 2)
plane_inv_tm(const TileDesc* __restrict__ tiles, const int2* __restrict__ items, const FftPlan* __restrict__ plans,
             const float2* __restrict__ spec, Epi epi, const __grid_constant__ EpiBoxes boxes) {
  constexpr int M = TX / 2, PX = M + 1, PITCH = fixed_pitch(TX), T = kTmThreads;
  constexpr SplitC sx = split_of(M), sy = split_of(TY);
  constexpr int EYMAX = tm_max_rows<TX, TY>();
  static_assert(sx.s == 2 && sy.s == 2 && !fixed_skew(TX), "two-stage lengths in the plain row layout");
  extern __shared__ float2 sm[];
  __shared__ uint32_t tslot;
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int z = it.y;
  if (threadIdx.x == 0)
    for (int i = 0; i < boxes.count; ++i) prefetch_box_l2(&boxes.map[i], (t.ox + t.hx) & ~3, t.oy + t.hy, t.oz + z);
  if (threadIdx.x < 32) tc::tmem_alloc(&tslot, kTmCols);
  float2* a = sm;
  const FftPlan* pxp = plans + t.plan_x;
  const float2* twx = pxp->tw;
  const float2* twy = plans[t.plan_y].tw;
  // y stage 0 straight from the spectrum slice into the buffer
  SpecSliceLoad ld{spec + t.spec_off + (long long)z * TY * PX, PX};
  stage_c<sy.r[0], TY, 1, true, false, T>(PX, twy, ld, SmemC<PITCH, 1, false>{a});
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tcol = tm_thread_col(tslot);
  stage_staged<sy.r[1], TY, sy.r[0], true, T, ceil_div(PX * (TY / sy.r[1]), T)>(
      PX, twy, SmemC<PITCH, 1, false>{a}, SmemC<PITCH, 1, false>{a}, tcol);
  // the effective rows: C2R along x, both stages in place
  float2* rows = a + t.hy * PITCH;
  stage_staged<sx.r[0], M, 1, true, T, ceil_div(EYMAX * (M / sx.r[0]), T)>(
      t.ey, twx, C2RRowLoad{rows, PITCH, M, pxp->tw_r2c}, SmemC<1, PITCH, false>{rows}, tcol);
  stage_staged<sx.r[1], M, sx.r[0], true, T, ceil_div(EYMAX * (M / sx.r[1]), T)>(
      t.ey, twx, SmemC<1, PITCH, false>{rows}, SmemC<1, PITCH, false>{rows}, tcol);
  if (threadIdx.x < 32) tc::tmem_dealloc(tslot, kTmCols);
  // the epilogue walks the effective region by whole warps per row (as plane_inv_fixed)
  const float* f = reinterpret_cast<const float*>(rows) + t.hx;
  const long long gz = t.oz + z;
  const int lane = threadIdx.x & 31;
  epi.acc_init();
  for (int row = threadIdx.x >> 5; row < t.ey; row += T / 32) {
    const long long g0 = (gz * epi.ny + (t.oy + t.hy + row)) * (long long)epi.nx + t.ox + t.hx;
    const float* srow = f + row * (2 * PITCH);
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
        val[u] = ok[u] ? srow[x] : 0.f;
      }
      epi.template apply<U>(g0, off, val, ok);
    }
  }
  epi.finish();
}

// Shapes (x length, y length) with in-place kernels: the large compiled planes.
#define MVD_TM_PLANE_SHAPES(X) \
  X(160, 160)                  \
  X(192, 96)                   \
  X(192, 135)

}  // namespace mvd
