// Instantiations and launches of the z-pencil pass (split from engine.cu so the library builds in parallel).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "engine.h"
#include "fixed_plane.cuh"
#include "zpass_tc.cuh"

namespace mvd {

// Occupancy variant of the z pass: registers sized for three CTAs per SM (measured faster);
// MVD_ZOCC=2 selects the two-CTA variant.
static int z_occupancy() {
  static int occ = [] {
    const char* e = std::getenv("MVD_ZOCC");
    return (e && std::atoi(e) == 2) ? 2 : 3;
  }();
  return occ;
}

// The in-place z pass (zpass_ip, kZWideChunk pencils per CTA) for the compiled two-stage
// lengths; MVD_Z_INPLACE=0 selects the two-buffer kernel.
static bool z_in_place() {
  static bool on = [] {
    const char* e = std::getenv("MVD_Z_INPLACE");
    return !(e && e[0] == '0');
  }();
  return on;
}

// The compile-time-length z pass for the plan's pencil length, if one is compiled.
static bool launch_z_fixed(PlanTable& pt, const ConvPlan& p, float2* spec, const float2* otf, cudaStream_t s) {
  if (p.generic || !use_fixed_planes() || z_occupancy() != 3) return false;
  const int tz = p.az.T;
#define MVD_Z_CASE(TZ)                                                                                       \
  if (tz == TZ) {                                                                                            \
    if (z_in_place()) {                                                                                      \
      constexpr int NT = zpass_ip_threads(TZ);                                                               \
      auto k = zpass_ip<TZ, kZWideChunk, NT, 2>;                                                             \
      const size_t sm = (size_t)TZ * (kZWideChunk + 1) * sizeof(float2);                                     \
      set_smem(k, sm);                                                                                       \
      k<<<(int)p.items_zw.size(), NT, sm, s>>>(p.d_tiles.as<TileDesc>(), p.d_items_zw.as<int2>(),           \
                                               pt.device(), spec, otf);                                     \
      return true;                                                                                           \
    }                                                                                                        \
    auto k = zpass_fixed<TZ, zpass_fixed_occ(TZ)>;                                                         \
    set_smem(k, p.smem_z);                                                                                   \
    k<<<(int)p.items_z.size(), kZThreads, p.smem_z, s>>>(p.d_tiles.as<TileDesc>(), p.d_items_z.as<int2>(), \
                                                          pt.device(), spec, otf);                          \
    return true;                                                                                             \
  }
  MVD_FIXED_Z_LENGTHS(MVD_Z_CASE)
#undef MVD_Z_CASE
  return false;
}

namespace {

// Per-device state of the tensor-core z pass: the 16-point DFT matrices (forward and inverse,
// each split into TF32 hi and lo parts) in the operand layout, and the count of waits that gave
// up.  Both live for the process.
struct TcState {
  float4* mats = nullptr;
  int* failures = nullptr;
};

TcState& tc_state() {
  static std::mutex mu;
  static std::vector<TcState> states;
  int dev = 0;
  MVD_CHECK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if ((int)states.size() <= dev) states.resize(dev + 1);
  TcState& st = states[dev];
  if (!st.mats) {
    // B[k][n] of the real form of y_q = sum_r x_r W^(r q), k = 2 r + c (c: real / imaginary part of
    // x_r), n = 2 q + d; W = exp(-+2 pi i / 16).  Stored transposed (row n, column k) in the
    // unswizzled K-major layout, as hi (the TF32 part: low 13 bits cleared) and lo = W - hi.
    std::vector<float> host(kTcMats * kTcK * kTcK, 0.f);
    for (int inv = 0; inv < 2; ++inv)
      for (int n = 0; n < kTcK; ++n)
        for (int k = 0; k < kTcK; ++k) {
          const int q = n / 2, d = n % 2, r = k / 2, c = k % 2;
          const double a = (inv ? 2.0 : -2.0) * M_PI * (double)((r * q) % 16) / 16.0;
          const double wre = std::cos(a), wim = std::sin(a);
          const double val = c == 0 ? (d == 0 ? wre : wim) : (d == 0 ? -wim : wre);
          float f = (float)val;
          uint32_t bits;
          std::memcpy(&bits, &f, 4);
          bits &= 0xFFFFE000u;
          float hi;
          std::memcpy(&hi, &bits, 4);
          const float lo = (float)(val - (double)hi);
          const size_t off = tc::kmajor_offset(n, k, kTcK) / 4;
          host[(2 * inv + 0) * kTcK * kTcK + off] = hi;
          host[(2 * inv + 1) * kTcK * kTcK + off] = lo;
        }
    MVD_CHECK(cudaMalloc(&st.mats, host.size() * sizeof(float)));
    MVD_CHECK(cudaMemcpy(st.mats, host.data(), host.size() * sizeof(float), cudaMemcpyHostToDevice));
    MVD_CHECK(cudaMalloc(&st.failures, sizeof(int)));
    MVD_CHECK(cudaMemset(st.failures, 0, sizeof(int)));
  }
  return st;
}

// Polls of each bounded MMA wait: 2^22 (far beyond a product's microseconds), or
// MVD_TC_WAIT_POLLS (>= 0) -- 0 makes every wait give up at once, which is how the failure path
// (error count, bounded wait for the products in flight, tensor memory freed) is tested.
int tc_wait_polls() {
  static int polls = [] {
    const char* e = std::getenv("MVD_TC_WAIT_POLLS");
    return (e && *e) ? std::max(0, std::atoi(e)) : (1 << 22);
  }();
  return polls;
}

// The tensor-core z pass for the plan's pencil length, if it has one.
bool launch_z_tc(PlanTable& pt, const ConvPlan& p, float2* spec, const float2* otf, cudaStream_t s) {
  const int tz = p.az.T;
#define MVD_TC_CASE(TZ)                                                                                       \
  if (tz == TZ) {                                                                                             \
    TcState& st = tc_state();                                                                                 \
    auto k = zpass_tc<TZ>;                                                                                    \
    const size_t sm = zpass_tc_smem<TZ>();                                                                    \
    set_smem(k, sm);                                                                                          \
    k<<<(int)p.items_z.size(), kZThreads, sm, s>>>(p.d_tiles.as<TileDesc>(), p.d_items_z.as<int2>(), pt.device(), \
                                                   spec, otf, st.mats, st.failures, tc_wait_polls());         \
    return true;                                                                                              \
  }
  MVD_TC_Z_LENGTHS(MVD_TC_CASE)
#undef MVD_TC_CASE
  return false;
}

}  // namespace

void tensor_dft_prepare() { tc_state(); }

bool tensor_dft_supported(int tz) {
#define MVD_TC_LEN(TZ) if (tz == TZ) return true;
  MVD_TC_Z_LENGTHS(MVD_TC_LEN)
#undef MVD_TC_LEN
  return false;
}

int tensor_dft_failures() {
  TcState& st = tc_state();
  int n = 0;
  MVD_CHECK(cudaMemcpy(&n, st.failures, sizeof(int), cudaMemcpyDeviceToHost));
  if (n) MVD_CHECK(cudaMemset(st.failures, 0, sizeof(int)));
  return n;
}

void launch_z(PlanTable& pt, const ConvPlan& p, float2* spec, const float2* otf, cudaStream_t s) {
  if (p.items_z.empty()) return;
  if (p.tensor_dft && !p.generic && launch_z_tc(pt, p, spec, otf, s)) {
    MVD_CHECK(cudaGetLastError());
    count_launch();
    return;
  }
  if (launch_z_fixed(pt, p, spec, otf, s)) {
    MVD_CHECK(cudaGetLastError());
    count_launch();
    return;
  }
  auto k = z_occupancy() == 3 ? zpass_kernel<0, 3> : zpass_kernel<0, 2>;
  set_smem(k, p.smem_z);
  k<<<(int)p.items_z.size(), kZThreads, p.smem_z, s>>>(p.d_tiles.as<TileDesc>(), p.d_items_z.as<int2>(), pt.device(),
                                                        spec, otf, 1.f);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

void launch_z_forward_scaled(PlanTable& pt, const ConvPlan& p, const TileDesc* tiles, const int2* items, int nitems,
                             float2* spec, float scale, cudaStream_t s) {
  if (nitems == 0) return;
  auto k = zpass_kernel<1>;
  set_smem(k, p.smem_z);
  k<<<nitems, kZThreads, p.smem_z, s>>>(tiles, items, pt.device(), spec, nullptr, scale);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

void launch_z_forward(PlanTable& pt, const ConvPlan& p, float2* spec, cudaStream_t s) {
  launch_z_forward_scaled(pt, p, p.d_tiles.as<TileDesc>(), p.d_items_z.as<int2>(), (int)p.items_z.size(), spec, 1.f, s);
}

void launch_z_inverse_items(PlanTable& pt, const ConvPlan& p, const TileDesc* tiles, const int2* items, int nitems,
                            float2* spec, cudaStream_t s) {
  if (nitems == 0) return;
  auto k = zpass_kernel<2>;
  set_smem(k, p.smem_z);
  k<<<nitems, kZThreads, p.smem_z, s>>>(tiles, items, pt.device(), spec, nullptr, 1.f);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

}  // namespace mvd
