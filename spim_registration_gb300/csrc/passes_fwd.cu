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
#include "fixed_plane_tm.cuh"

namespace mvd {

namespace {

// CTAs of a plane kernel resident at once on the current device
int resident_ctas(int per_sm) {
  int dev = 0, sms = 0;
  MVD_CHECK(cudaGetDevice(&dev));
  MVD_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  return per_sm * sms;
}

}  // namespace

// The compile-time-shaped kernel for (tx, ty), if one is compiled (plans at the default CTA
// size run it at its own size).
template <class Gather>
static bool launch_fwd_fixed(int tx, int ty, int threads, PlanTable& pt, const TileDesc* tiles, const int2* items,
                             int nitems, size_t smem, float2* spec, Gather g, cudaStream_t s, bool staged) {
  if (threads != kThreads || !use_fixed_planes()) return false;
  if (staged) {
#define MVD_FWD_TM_CASE(TX, TY)                                                                         \
    if (tx == TX && ty == TY) {                                                                         \
      EpiBoxes src;                                                                                     \
      std::memset(&src, 0, sizeof(src));                                                                \
      src.count = use_l2_prefetch() &&                                                                  \
                  volume_box_map(g.v.data, g.v.nx, g.v.ny, g.v.nz, prefetch_box_width(TX), TY, &src.map[0]); \
      auto k = plane_fwd_tm<Gather, TX, TY>;                                                            \
      const size_t sm = (size_t)TY * fixed_pitch(TX) * sizeof(float2);                                  \
      set_smem(k, sm);                                                                                  \
      k<<<nitems, kTmThreads, sm, s>>>(tiles, items, pt.device(), spec, g, src, resident_ctas(2));      \
      return true;                                                                                      \
    }
    MVD_TM_PLANE_SHAPES(MVD_FWD_TM_CASE)
#undef MVD_FWD_TM_CASE
  }
#define MVD_FWD_CASE(TX, TY, T)                                                                         \
  if (tx == TX && ty == TY) {                                                                           \
    EpiBoxes src;                                                                                       \
    std::memset(&src, 0, sizeof(src));                                                                  \
    src.count = use_l2_prefetch() &&                                                                    \
                volume_box_map(g.v.data, g.v.nx, g.v.ny, g.v.nz, prefetch_box_width(TX), TY, &src.map[0]); \
    auto k = plane_fwd_fixed<Gather, TX, TY, T>;                                                        \
    set_smem(k, smem);                                                                                  \
    k<<<nitems, T, smem, s>>>(tiles, items, pt.device(), spec, g, src, resident_ctas(fixed_ctas_per_sm(TX, TY))); \
    return true;                                                                                        \
  }
  MVD_FIXED_PLANE_SHAPES(MVD_FWD_CASE)
#undef MVD_FWD_CASE
  return false;
}

bool compiled_plane_shape(int tx, int ty) {
#define MVD_SHAPE_Q(SX, SY, ST) \
  if (tx == SX && ty == SY) return true;
  MVD_FIXED_PLANE_SHAPES(MVD_SHAPE_Q)
#undef MVD_SHAPE_Q
  return false;
}

int compiled_plane_threads(const ConvPlan& p) {
#define MVD_SHAPE_T(SX, SY, ST) \
  if (p.ax.T == SX && p.ay.T == SY) return ST;
  MVD_FIXED_PLANE_SHAPES(MVD_SHAPE_T)
#undef MVD_SHAPE_T
  return 0;
}

bool staged_plane_shape(int tx, int ty) {
#define MVD_TM_S(SX, SY) \
  if (tx == SX && ty == SY) return true;
  MVD_TM_PLANE_SHAPES(MVD_TM_S)
#undef MVD_TM_S
  return false;
}

bool has_staged_kernels(const ConvPlan& p) {
#define MVD_TM_Q(SX, SY) \
  if (p.ax.T == SX && p.ay.T == SY) return p.ay.E <= tm_max_rows<SX, SY>();
  MVD_TM_PLANE_SHAPES(MVD_TM_Q)
#undef MVD_TM_Q
  return false;
}

bool has_compiled_kernels(const ConvPlan& p) {
  if (compiled_plane_threads(p)) return true;
#define MVD_Z_LEN(SZ) \
  if (p.az.T == SZ) return true;
  MVD_FIXED_Z_LENGTHS(MVD_Z_LEN)
#undef MVD_Z_LEN
  return false;
}

template <class Gather, bool MASK = false>
static void launch_fwd_impl(PlanTable& pt, const TileDesc* tiles, const int2* items, int nitems, size_t smem,
                            int threads, int tx, int ty, float2* spec, Gather g, cudaStream_t s,
                            bool generic = false, bool staged = false) {
  if (nitems == 0) return;
  if (MASK || generic ||
      !launch_fwd_fixed(tx, ty, threads > 0 ? threads : kThreads, pt, tiles, items, nitems, smem, spec, g, s,
                        staged)) {
    EpiBoxes src;
    std::memset(&src, 0, sizeof(src));
    src.count = !MASK && use_l2_prefetch() &&
                volume_box_map(g.v.data, g.v.nx, g.v.ny, g.v.nz, prefetch_box_width(tx), ty, &src.map[0]);
    auto k = plane_fwd_kernel<Gather, MASK>;
    set_smem(k, smem);
    const int per_sm = 2 * smem <= 200 * 1024 ? 2 : 1;  // CTAs of this size an SM holds at once
    k<<<nitems, threads > 0 ? threads : kThreads, smem, s>>>(tiles, items, pt.device(), spec, g, src,
                                                             resident_ctas(per_sm));
  }
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

void launch_fwd_mirror(PlanTable& pt, const ConvPlan& p, const float* vol, float2* spec, cudaStream_t s) {
  GatherMirror g{{vol, p.vol[0], p.vol[1], p.vol[2]}};
  launch_fwd_impl(pt, p.d_tiles.as<TileDesc>(), p.d_items_fwd.as<int2>(), (int)p.items_fwd.size(), p.smem_plane,
                  p.threads_plane, p.ax.T, p.ay.T, spec, g, s, p.generic, p.staged);
}

void launch_fwd_value(PlanTable& pt, const ConvPlan& p, const float* vol, float value, float2* spec,
                      cudaStream_t s) {
  GatherValue g = GatherValue::box(vol, p.vol[0], p.vol[1], p.vol[2], value, p.box_lo[0], p.box_lo[1], p.box_lo[2],
                                   p.box_hi[0], p.box_hi[1], p.box_hi[2]);
  launch_fwd_impl(pt, p.d_tiles.as<TileDesc>(), p.d_items_fwd.as<int2>(), (int)p.items_fwd.size(), p.smem_plane,
                  p.threads_plane, p.ax.T, p.ay.T, spec, g, s, p.generic, p.staged);
}

void launch_fwd_value_items(PlanTable& pt, const ConvPlan& p, const TileDesc* tiles, const int2* items, int nitems,
                            const float* vol, int vx, int vy, int vz, float value, float2* spec, cudaStream_t s) {
  GatherValue g = GatherValue::full(vol, vx, vy, vz, value);
  launch_fwd_impl(pt, tiles, items, nitems, p.smem_plane, p.threads_plane, p.ax.T, p.ay.T, spec, g, s, p.generic);
}

void launch_fwd_masked(PlanTable& pt, const ConvPlan& p, const float* vol, float2* spec, cudaStream_t s) {
  GatherValue g = GatherValue::full(vol, p.vol[0], p.vol[1], p.vol[2], 0.f);
  launch_fwd_impl<GatherValue, true>(pt, p.d_tiles.as<TileDesc>(), p.d_items_fwd.as<int2>(), (int)p.items_fwd.size(),
                                     p.smem_plane, p.threads_plane, p.ax.T, p.ay.T, spec, g, s);
}

}  // namespace mvd
