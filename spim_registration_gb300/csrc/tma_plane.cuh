// Forward plane pass with the tile slice brought into shared memory by the Tensor Memory
// Accelerator (cp.async.bulk.tensor), for the compile-time tile shapes.
//
// The generic first row stage gathers the slice straight from the volume, j-fastest: a warp's
// loads cover only N/R0 consecutive pairs of a row, so the gather costs about 3.7x the L1
// sectors of one coalesced read and keeps the L1/shared pipe near saturation.  Here one thread
// issues a single 3D TMA copy of the slice's box [x0, x0 + W) x [oy, oy + TY) x {z} into shared
// memory (x0 = ox rounded down to a multiple of 4 floats: a tensor copy must start on a 16-byte
// boundary; the tile's x = 0 sits at offset r0 = ox - x0 of each row).  Parts of the box
// outside the volume come back zero-filled; a warp-per-row fix-up then rewrites every
// position outside the gather's region (the volume for the mirror-single rule, the data box for
// the value rule) through the gather functor itself, so the slice is exactly what the generic
// gather reads.  The first row stage then reads the slice from shared memory.  The slice buffer
// is reused as the second ping-pong buffer, so the kernel fits two CTAs per SM.
//
// The copy completes on an mbarrier; the wait is bounded: if it gives up, the CTA records the
// timeout in a device flag, waits (bounded) for the copy once more and returns without
// computing.
#pragma once
#include <cuda.h>  // CUtensorMap

#include "fixed_plane.cuh"

namespace mvd {
namespace tma {

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n"
      "  .reg .pred p;\n"
      "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "  selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// bounded wait for phase `parity` of the barrier
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  for (int i = 0; i < (1 << 20); ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void load_box_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

}  // namespace tma

// First row stage's loads from the staged slice: packed pair n = (x[2n], x[2n+1]) of row `batch`.
struct StagedPairs {
  const float* s;  // row 0, tile-local x = 0
  int w;           // row pitch (floats)
  template <int R>
  __device__ __forceinline__ void get(int batch, int j, int NR, float2* v) const {
    const float* row = s + batch * w;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int x = 2 * (j + r * NR);
      v[r] = make_float2(row[x], row[x + 1]);
    }
  }
};

// Box width (floats) of the slice copy: the tile's TX columns at any offset r0 in [0, 4),
// rounded to 16 bytes.
__host__ __device__ constexpr int tma_box_width(int TX) { return (TX + 3 + 3) / 4 * 4; }

template <int TX, int TY>
constexpr size_t tma_plane_smem() {
  return (size_t)TY * tma_box_width(TX) * sizeof(float) + (size_t)TY * row_pitch(TX / 2) * sizeof(float2);
}

template <class Gather, int TX, int TY, int T>
__global__ void __launch_bounds__(T, 2)
plane_fwd_tma(const TileDesc* __restrict__ tiles, const int2* __restrict__ items, const FftPlan* __restrict__ plans,
              float2* __restrict__ spec, Gather gather, const __grid_constant__ CUtensorMap box_map, int* timeouts) {
  constexpr int M = TX / 2, PX = M + 1, PITCH = row_pitch(M), P1 = M + 1, W = tma_box_width(TX);
  static_assert(P1 % 2 == 1, "the stage-1 pitch must be odd (conflict-free batch-fastest access)");
  constexpr SplitC sx = split_of(M), sy = split_of(TY);
  static_assert(sx.s == 2 && sy.s == 2, "two-stage row and column transforms");
  extern __shared__ __align__(1024) unsigned char smraw[];
  float* S = reinterpret_cast<float*>(smraw);                                             // TY x W floats
  float2* cur = reinterpret_cast<float2*>(smraw + (size_t)TY * W * sizeof(float));         // TY x PITCH
  __shared__ __align__(8) uint64_t bar;
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int z = it.y;
  const int gz = t.oz + z;
  const int x0 = t.ox & ~3;  // rounds down for negative origins too
  const int r0 = t.ox - x0;
  int zsrc = 0;
  const bool load = gather.slice_source(gz, zsrc);
  if (threadIdx.x == 0) {
    tma::mbar_init(&bar, 1);
    tma::fence_mbar_init();
  }
  __syncthreads();
  if (load) {
    if (threadIdx.x == 0) {
      tma::mbar_expect_tx(&bar, (unsigned)(TY * W * sizeof(float)));
      tma::load_box_3d(S, &box_map, &bar, x0, t.oy, zsrc);
    }
    const bool ok = tma::mbar_wait(&bar, 0);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicAdd(timeouts, 1);
      tma::mbar_wait(&bar, 0);  // the copy may still land: wait once more before leaving
      return;
    }
  }
  // rewrite everything outside the gather's region (or the whole slice when nothing was copied)
  {
    int lox, hix, loy, hiy;
    gather.region(lox, hix, loy, hiy);
    const int lane = threadIdx.x & 31;
    const int xa = min(max(lox - t.ox, 0), TX), xb = min(max(hix - t.ox, 0), TX);
    for (int b = threadIdx.x >> 5; b < TY; b += T / 32) {
      const int gy = t.oy + b;
      const auto rg = gather.row(gy, gz);
      float* row = S + b * W + r0;
      if (!load || gy < loy || gy >= hiy) {
        for (int x = lane; x < TX; x += 32) row[x] = rg(t.ox + x);
      } else {
        for (int x = lane; x < xa; x += 32) row[x] = rg(t.ox + x);
        for (int x = xb + lane; x < TX; x += 32) row[x] = rg(t.ox + x);
      }
    }
  }
  __syncthreads();
  const FftPlan* pxp = plans + t.plan_x;
  const float2* twx = pxp->tw;
  // x stage 0: staged slice -> cur (skewed rows), j-fastest
  stage_c<sx.r[0], M, 1, false, true, T>(TY, twx, StagedPairs{S + r0, W}, SmemC<1, PITCH, true>{cur});
  __syncthreads();
  // x stage 1: cur -> the slice buffer, now rows of P1 complex
  float2* S2 = reinterpret_cast<float2*>(S);
  stage_c<sx.r[1], M, sx.r[0], false, false, T>(TY, twx, SmemC<1, PITCH, true>{cur}, SmemC<1, P1, false>{S2});
  __syncthreads();
  // y: half-spectrum columns formed while loading, then to the spectrum slice
  const float2* twy = plans[t.plan_y].tw;
  stage_c<sy.r[0], TY, 1, false, false, T>(PX, twy, R2CColumnLoad{S2, P1, M, pxp->tw_r2c},
                                           SmemC<PITCH, 1, false>{cur});
  __syncthreads();
  SpecSliceStore st{spec + t.spec_off + (long long)z * TY * PX, PX};
  stage_c<sy.r[1], TY, sy.r[0], false, false, T>(PX, twy, SmemC<PITCH, 1, false>{cur}, st);
}

}  // namespace mvd
