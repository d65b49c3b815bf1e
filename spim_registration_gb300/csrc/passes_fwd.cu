// Instantiations and launches of the forward plane pass (split from engine.cu so the library builds in parallel).
#include <cuda.h>

#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "engine.h"
#include "fixed_plane.cuh"
#include "tma_plane.cuh"

namespace mvd {

namespace {

// CTAs of a plane kernel resident at once on the current device (two per SM)
int resident_ctas() {
  int dev = 0, sms = 0;
  MVD_CHECK(cudaGetDevice(&dev));
  MVD_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  return 2 * sms;
}

// Per-device count of slice copies whose wait gave up (zero unless a copy never completed).
int* tma_timeout_counter() {
  static std::mutex mu;
  static std::vector<int*> ptrs;
  int dev = 0;
  MVD_CHECK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if ((int)ptrs.size() <= dev) ptrs.resize(dev + 1, nullptr);
  if (!ptrs[dev]) {
    MVD_CHECK(cudaMalloc(&ptrs[dev], sizeof(int)));
    MVD_CHECK(cudaMemset(ptrs[dev], 0, sizeof(int)));
  }
  return ptrs[dev];
}

}  // namespace

int tma_timeouts() {
  if (!use_tma()) return 0;
  int n = 0;
  MVD_CHECK(cudaMemcpy(&n, tma_timeout_counter(), sizeof(int), cudaMemcpyDeviceToHost));
  if (n) MVD_CHECK(cudaMemset(tma_timeout_counter(), 0, sizeof(int)));
  return n;
}

// The compile-time-shaped kernel for (tx, ty) at 384 threads, if one is compiled.
template <class Gather>
static bool launch_fwd_fixed(int tx, int ty, int threads, PlanTable& pt, const TileDesc* tiles, const int2* items,
                             int nitems, size_t smem, float2* spec, Gather g, cudaStream_t s) {
  if (threads != kThreads || !use_fixed_planes()) return false;
#define MVD_FWD_CASE(TX, TY)                                                                              \
  if (tx == TX && ty == TY) {                                                                             \
    CUtensorMap map;                                                                                      \
    if (use_tma() && volume_box_map(g.v.data, g.v.nx, g.v.ny, g.v.nz, tma_box_width(TX), TY, &map)) {     \
      auto k = plane_fwd_tma<Gather, TX, TY, kFixedThreads>;                                              \
      const size_t sm = tma_plane_smem<TX, TY>();                                                         \
      set_smem(k, sm);                                                                                    \
      k<<<nitems, kFixedThreads, sm, s>>>(tiles, items, pt.device(), spec, g, map, tma_timeout_counter()); \
    } else {                                                                                              \
      EpiBoxes src;                                                                                       \
      std::memset(&src, 0, sizeof(src));                                                                  \
      src.count = use_l2_prefetch() &&                                                                    \
                  volume_box_map(g.v.data, g.v.nx, g.v.ny, g.v.nz, tma_box_width(TX), TY, &src.map[0]);   \
      auto k = plane_fwd_fixed<Gather, TX, TY, kFixedThreads>;                                            \
      set_smem(k, smem);                                                                                  \
      k<<<nitems, kFixedThreads, smem, s>>>(tiles, items, pt.device(), spec, g, src, resident_ctas());    \
    }                                                                                                     \
    return true;                                                                                          \
  }
  MVD_FIXED_PLANE_SHAPES(MVD_FWD_CASE)
#undef MVD_FWD_CASE
  return false;
}

template <class Gather, bool MASK = false>
static void launch_fwd_impl(PlanTable& pt, const TileDesc* tiles, const int2* items, int nitems, size_t smem,
                            int threads, int tx, int ty, float2* spec, Gather g, cudaStream_t s) {
  if (nitems == 0) return;
  if (MASK || !launch_fwd_fixed(tx, ty, threads > 0 ? threads : kThreads, pt, tiles, items, nitems, smem, spec, g,
                                s)) {
    EpiBoxes src;
    std::memset(&src, 0, sizeof(src));
    src.count = !MASK && use_l2_prefetch() &&
                volume_box_map(g.v.data, g.v.nx, g.v.ny, g.v.nz, tma_box_width(tx), ty, &src.map[0]);
    auto k = plane_fwd_kernel<Gather, MASK>;
    set_smem(k, smem);
    k<<<nitems, threads > 0 ? threads : kThreads, smem, s>>>(tiles, items, pt.device(), spec, g, src, resident_ctas());
  }
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

void launch_fwd_mirror(PlanTable& pt, const ConvPlan& p, const float* vol, float2* spec, cudaStream_t s) {
  GatherMirror g{{vol, p.vol[0], p.vol[1], p.vol[2]}};
  launch_fwd_impl(pt, p.d_tiles.as<TileDesc>(), p.d_items_fwd.as<int2>(), (int)p.items_fwd.size(), p.smem_plane,
                  p.threads_plane, p.ax.T, p.ay.T, spec, g, s);
}

void launch_fwd_value(PlanTable& pt, const ConvPlan& p, const float* vol, float value, float2* spec,
                      cudaStream_t s) {
  GatherValue g = GatherValue::box(vol, p.vol[0], p.vol[1], p.vol[2], value, p.box_lo[0], p.box_lo[1], p.box_lo[2],
                                   p.box_hi[0], p.box_hi[1], p.box_hi[2]);
  launch_fwd_impl(pt, p.d_tiles.as<TileDesc>(), p.d_items_fwd.as<int2>(), (int)p.items_fwd.size(), p.smem_plane,
                  p.threads_plane, p.ax.T, p.ay.T, spec, g, s);
}

void launch_fwd_value_items(PlanTable& pt, const ConvPlan& p, const TileDesc* tiles, const int2* items, int nitems,
                            const float* vol, int vx, int vy, int vz, float value, float2* spec, cudaStream_t s) {
  GatherValue g = GatherValue::full(vol, vx, vy, vz, value);
  launch_fwd_impl(pt, tiles, items, nitems, p.smem_plane, p.threads_plane, p.ax.T, p.ay.T, spec, g, s);
}

void launch_fwd_masked(PlanTable& pt, const ConvPlan& p, const float* vol, float2* spec, cudaStream_t s) {
  GatherValue g = GatherValue::full(vol, p.vol[0], p.vol[1], p.vol[2], 0.f);
  launch_fwd_impl<GatherValue, true>(pt, p.d_tiles.as<TileDesc>(), p.d_items_fwd.as<int2>(), (int)p.items_fwd.size(),
                                     p.smem_plane, p.threads_plane, p.ax.T, p.ay.T, spec, g, s);
}

}  // namespace mvd
