// The z pass of a convolution with its inner DFT stage on the tensor cores (tcgen05, TF32 with
// FP32 accumulation, three-term split for FP32-level accuracy).
//
// For a pencil length TZ = R0 x 16 the SIMT z pass (zpass_fixed) runs the forward radix-R0 stage,
// then the fused middle stage -- forward radix-16 DFT, product with the kernel spectrum, inverse
// radix-16 DFT -- and finally the inverse radix-R0 stage.  Here the two 16-point DFTs of the
// middle stage are matrix products: the 16 pencils x TZ/16 butterflies of the CTA are the rows of
// A (16 complex inputs as 32 interleaved reals per row, after the stage's twiddles) and the
// 16-point DFT is a real 32x32 matrix B, so Y = A B on the tensor core, 128 rows per product.
// Each operand is split as x = hi + lo (hi keeps the 10 mantissa bits a TF32 operand holds, lo the
// next 11), and A B = A_hi B_hi + A_lo B_hi + A_hi B_lo accumulates in FP32 in tensor memory: the
// dropped A_lo B_lo term and the truncation of lo leave a relative error near 2^-21 per product.
// Results are read back with tcgen05.ld (one butterfly row per thread and 8 complex values per
// half of the CTA), multiplied by the kernel spectrum in registers and fed to the inverse product.
//
// `polls` bounds every wait (the host passes 2^22, or MVD_TC_WAIT_POLLS for the failure test).
// The CTA: 256 threads, one CTA per SM (the operand tiles take 48 KB of shared memory on top of
// the two pencil buffers), 64 tensor-memory columns (forward and inverse accumulators).  Every
// wait on the MMA completion is bounded; a wait that gives up records it in `err`, skips the
// rest of the CTA's work (its pencils are then wrong, and the host reports the error), waits once
// more (bounded) for the products in flight and frees the tensor memory before returning.
#pragma once
#include "fixed_plane.cuh"
#include "tcgen05.cuh"

namespace mvd {

constexpr int kTcRows = 128;                         // rows of one MMA tile (M)
constexpr int kTcK = 32;                             // 16 complex values as 32 reals (K = N = 32)
constexpr int kTcOperandBytes = kTcRows * kTcK * 4;  // one A tile (16 KB)
constexpr int kTcMatBytes = kTcK * kTcK * 4;         // one B matrix (4 KB)
// B matrices in the operand layout, in this order: forward hi, forward lo, inverse hi, inverse lo
constexpr int kTcMats = 4;

template <int TZ>
__host__ __device__ constexpr size_t zpass_tc_smem() {
  return 2 * (size_t)TZ * kZPitch * sizeof(float2) + 2 * kTcOperandBytes + kTcMats * kTcMatBytes;
}

template <int TZ>
__global__ void __launch_bounds__(kZThreads, 1)
zpass_tc(const TileDesc* __restrict__ tiles, const int2* __restrict__ items, const FftPlan* __restrict__ plans,
         float2* __restrict__ spec, const float2* __restrict__ otf, const float4* __restrict__ dft_mats, int* err,
         int polls) {
  constexpr SplitC sp = split_of(TZ);
  static_assert(sp.s == 2 && sp.r[1] == 16, "tensor-core middle stage needs TZ = R0 x 16");
  constexpr int R0 = sp.r[0];
  constexpr int NR = TZ / 16;  // butterflies of the middle stage per pencil
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // operand tiles first, then the B matrices, then the pencil buffers (all 16-byte aligned, as
  // the descriptors of unswizzled operands require)
  unsigned char* base = smem_raw;
  float* a_hi = reinterpret_cast<float*>(base);
  float* a_lo = reinterpret_cast<float*>(base + kTcOperandBytes);
  unsigned char* mats = base + 2 * kTcOperandBytes;
  float2* cur = reinterpret_cast<float2*>(mats + kTcMats * kTcMatBytes);
  float2* oth = cur + TZ * kZPitch;
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;

  const int tid = threadIdx.x;
  const int2 it = items[blockIdx.x];
  const TileDesc t = tiles[it.x];
  const int p0 = it.y;
  const int plane = t.ty * t.px;
  const int count = min(kZChunk, plane - p0);
  const float2* tw = plans[t.plan_z].tw;
  PencilRef g{spec + t.spec_off + p0, plane};
  const float2* otf_p = otf + t.otf_off + p0;

  // set-up: the DFT matrices into shared memory, the mbarrier, 64 tensor-memory columns
  {
    float4* dst = reinterpret_cast<float4*>(mats);
    for (int i = tid; i < kTcMats * kTcMatBytes / 16; i += kZThreads) dst[i] = __ldg(dft_mats + i);
  }
  if (tid == 0) tc::mbar_init(&bar, 1);
  if (tid < 32) tc::tmem_alloc(&tslot, 64);
  // forward stage 0 straight from the pencils (SIMT)
  stage_c<R0, TZ, 1, false, false, kZThreads>(count, tw, g, SmemC<kZPitch, 1, false>{cur});
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot;
  const uint32_t d_fwd = tmem, d_inv = tmem + 32;
  const uint32_t idesc = tc::idesc_tf32(kTcRows, kTcK);
  const uint32_t a_addr[2] = {tc::smem_u32(a_hi), tc::smem_u32(a_lo)};
  const uint32_t b_addr = tc::smem_u32(mats);

  // this thread's row of every tile and its half of the row's 16 complex values
  const int row = tid & (kTcRows - 1);
  const int half = tid >> 7;  // values [8 half, 8 half + 8)
  const int nb = count * NR;
  uint32_t phase = 0;
  bool failed = false;

  // A operand rows: 8 complex values of this thread's half, split into hi and lo
  auto put_row = [&](const float2* v) {
#pragma unroll
    for (int q = 0; q < 8; q += 2) {  // two complex values = four reals = one 16-byte chunk
      const int k = 2 * (8 * half + q);
      float h[4], l[4];
      tc::split_tf32(v[q].x, h[0], l[0]);
      tc::split_tf32(v[q].y, h[1], l[1]);
      tc::split_tf32(v[q + 1].x, h[2], l[2]);
      tc::split_tf32(v[q + 1].y, h[3], l[3]);
      const uint32_t off = tc::kmajor_offset(row, k, kTcK);
      *reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(a_hi) + off) = make_float4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(a_lo) + off) = make_float4(l[0], l[1], l[2], l[3]);
    }
  };
  // one 16-point DFT of all 128 rows: three products per K step into the accumulator at d
  auto product = [&](uint32_t d, int mat_hi) {
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const int ai[3] = {0, 1, 0}, bi[3] = {0, 0, 1};
#pragma unroll
      for (int term = 0; term < 3; ++term)
#pragma unroll
        for (int kk = 0; kk < kTcK / 8; ++kk) {
          const uint64_t ad = tc::smem_desc(a_addr[ai[term]] + kk * 256, 128, 32 * kTcK);
          const uint64_t bd = tc::smem_desc(b_addr + (mat_hi + bi[term]) * kTcMatBytes + kk * 256, 128, 32 * kTcK);
          tc::mma_tf32(d, ad, bd, idesc, term > 0 || kk > 0);
        }
      tc::mma_commit(&bar);
    }
    const bool ok = tc::mbar_wait(&bar, phase, polls);
    phase ^= 1u;
    tc::fence_after_sync();
    return ok;
  };
  // this thread's 8 complex results of its row (lane quadrant = warp % 4 = row / 32)
  auto get_row = [&](uint32_t d, float2* v) {
    float r[16];
    tc::tmem_ld16(d + ((uint32_t)(row & ~31) << 16) + 16 * half, r);
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = make_float2(r[2 * q], r[2 * q + 1]);
  };

  for (int m0 = 0; m0 < nb && !failed; m0 += kTcRows) {
    const int b = m0 + row;
    const bool live = b < nb;
    const int j = live ? b / count : 0;
    const int batch = live ? b - j * count : 0;
    float2 v[8];
    if (live) {
      // inputs j + r NR of the butterfly, twiddled by w^(r j) (the forward last stage's twiddles)
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int r = 8 * half + q;
        float2 x = cur[batch + (j + r * NR) * kZPitch];
        if (j != 0 && r != 0) x = cmul(x, __ldg(tw + r * j));
        v[q] = x;
      }
    } else {
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = make_float2(0.f, 0.f);
    }
    put_row(v);
    failed = __syncthreads_or(!product(d_fwd, 0));
    if (failed) break;
    get_row(d_fwd, v);
    if (live) {  // product with the kernel spectrum at the natural index j + r NR
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = cmul(v[q], __ldg(otf_p + (j + (8 * half + q) * NR) * plane + batch));
    }
    put_row(v);
    failed = __syncthreads_or(!product(d_inv, 2));
    if (failed) break;
    get_row(d_inv, v);
    if (live) {  // the inverse first stage's Stockham order: element j 16 + r
#pragma unroll
      for (int q = 0; q < 8; ++q) oth[batch + (j * 16 + 8 * half + q) * kZPitch] = v[q];
    }
    tc::fence_before_sync();
  }
  if (failed) {
    if (tid == 0) atomicAdd(err, 1);
    tc::mbar_wait(&bar, phase ^ 1u, 1 << 20);  // the products of the wait that gave up (bounded)
  } else {
    __syncthreads();
    float2* c2 = oth;
    float2* o2 = cur;
    z_inv_stages<TZ, 1, kZThreads>(count, tw, PencilEffectiveStore{g.p, plane, t.hz, t.hz + t.ez}, c2, o2);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) tc::tmem_dealloc(tmem, 64);
}

// Pencil lengths with a tensor-core z pass (the 512x512x256 workload's).
#define MVD_TC_Z_LENGTHS(X) \
  X(320)                    \
  X(288)

}  // namespace mvd
