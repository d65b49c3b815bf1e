// Instantiations and launches of the z-pencil pass (split from engine.cu so the library builds in parallel).
#include <cstdlib>

#include "engine.h"
#include "fixed_plane.cuh"

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

// The compile-time-length z pass for the plan's pencil length, if one is compiled.
static bool launch_z_fixed(PlanTable& pt, const ConvPlan& p, float2* spec, const float2* otf, cudaStream_t s) {
  if (!use_fixed_planes() || z_occupancy() != 3) return false;
  const int tz = p.az.T;
#define MVD_Z_CASE(TZ)                                                                                       \
  if (tz == TZ) {                                                                                            \
    auto k = zpass_fixed<TZ, zpass_fixed_occ(TZ)>;                                                                           \
    set_smem(k, p.smem_z);                                                                                   \
    k<<<(int)p.items_z.size(), kZThreads, p.smem_z, s>>>(p.d_tiles.as<TileDesc>(), p.d_items_z.as<int2>(), \
                                                          pt.device(), spec, otf);                          \
    return true;                                                                                             \
  }
  MVD_FIXED_Z_LENGTHS(MVD_Z_CASE)
#undef MVD_Z_CASE
  return false;
}

void launch_z(PlanTable& pt, const ConvPlan& p, float2* spec, const float2* otf, cudaStream_t s) {
  if (p.items_z.empty()) return;
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
