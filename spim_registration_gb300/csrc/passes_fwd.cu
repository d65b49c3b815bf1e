// Instantiations and launches of the forward plane pass (split from engine.cu so the library builds in parallel).
#include "engine.h"

namespace mvd {

template <class Gather, bool MASK = false>
static void launch_fwd_impl(PlanTable& pt, const TileDesc* tiles, const int2* items, int nitems, size_t smem,
                            int threads, float2* spec, Gather g, cudaStream_t s) {
  if (nitems == 0) return;
  auto k = plane_fwd_kernel<Gather, MASK>;
  set_smem(k, smem);
  k<<<nitems, threads > 0 ? threads : kThreads, smem, s>>>(tiles, items, pt.device(), spec, g);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

void launch_fwd_mirror(PlanTable& pt, const ConvPlan& p, const float* vol, float2* spec, cudaStream_t s) {
  GatherMirror g{{vol, p.vol[0], p.vol[1], p.vol[2]}};
  launch_fwd_impl(pt, p.d_tiles.as<TileDesc>(), p.d_items_fwd.as<int2>(), (int)p.items_fwd.size(), p.smem_plane,
                  p.threads_plane, spec, g, s);
}

void launch_fwd_value(PlanTable& pt, const ConvPlan& p, const float* vol, float value, float2* spec,
                      cudaStream_t s) {
  GatherValue g = GatherValue::box(vol, p.vol[0], p.vol[1], p.vol[2], value, p.box_lo[0], p.box_lo[1], p.box_lo[2],
                                   p.box_hi[0], p.box_hi[1], p.box_hi[2]);
  launch_fwd_impl(pt, p.d_tiles.as<TileDesc>(), p.d_items_fwd.as<int2>(), (int)p.items_fwd.size(), p.smem_plane,
                  p.threads_plane, spec, g, s);
}

void launch_fwd_value_items(PlanTable& pt, const ConvPlan& p, const TileDesc* tiles, const int2* items, int nitems,
                            const float* vol, int vx, int vy, int vz, float value, float2* spec, cudaStream_t s) {
  GatherValue g = GatherValue::full(vol, vx, vy, vz, value);
  launch_fwd_impl(pt, tiles, items, nitems, p.smem_plane, p.threads_plane, spec, g, s);
}

void launch_fwd_masked(PlanTable& pt, const ConvPlan& p, const float* vol, float2* spec, cudaStream_t s) {
  GatherValue g = GatherValue::full(vol, p.vol[0], p.vol[1], p.vol[2], 0.f);
  launch_fwd_impl<GatherValue, true>(pt, p.d_tiles.as<TileDesc>(), p.d_items_fwd.as<int2>(), (int)p.items_fwd.size(),
                                     p.smem_plane, p.threads_plane, spec, g, s);
}

}  // namespace mvd
