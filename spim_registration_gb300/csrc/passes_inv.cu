// Instantiations and launches of the inverse plane pass (split from engine.cu so the library builds in parallel).
#include <cstdlib>
#include <cstring>

#include "engine.h"
#include "fixed_plane.cuh"
#include "fixed_plane_tm.cuh"

namespace mvd {

// Tensor maps for the L2 prefetch of the volumes the epilogue reads (none if any is refused).
template <class Epi>
static EpiBoxes epilogue_boxes(const ConvPlan& p, const Epi& e) {
  EpiBoxes b;
  std::memset(&b, 0, sizeof(b));
  const float* in[2] = {nullptr, nullptr};
  const int n = use_l2_prefetch() ? e.inputs(in) : 0;
  const int w = (p.ax.E + 3 + 3) / 4 * 4;
  for (int i = 0; i < n; ++i)
    if (!volume_box_map(in[i], p.vol[0], p.vol[1], p.vol[2], w, p.ay.E, &b.map[i])) return EpiBoxes{};
  b.count = n;
  return b;
}

// The compile-time-shaped kernel for the plan's tile shape, if one is compiled (plans at the
// default CTA size run it at its own size).
template <class Epi>
static bool launch_inv_fixed(PlanTable& pt, const ConvPlan& p, const TileDesc* tiles, const int2* items, int nitems,
                             const float2* spec, Epi e, cudaStream_t s) {
  const int threads = p.threads_plane > 0 ? p.threads_plane : kThreads;
  if (threads != kThreads || p.generic || !use_fixed_planes()) return false;
  const int tx = p.ax.T, ty = p.ay.T;
  const EpiBoxes boxes = epilogue_boxes(p, e);
  if (p.staged && has_staged_kernels(p)) {
#define MVD_INV_TM_CASE(TX, TY)                                                        \
    if (tx == TX && ty == TY) {                                                        \
      auto k = plane_inv_tm<Epi, TX, TY>;                                              \
      const size_t sm = (size_t)TY * fixed_pitch(TX) * sizeof(float2);                 \
      set_smem(k, sm);                                                                 \
      k<<<nitems, kTmThreads, sm, s>>>(tiles, items, pt.device(), spec, e, boxes);     \
      return true;                                                                     \
    }
    MVD_TM_PLANE_SHAPES(MVD_INV_TM_CASE)
#undef MVD_INV_TM_CASE
  }
#define MVD_INV_CASE(TX, TY, T)                                                        \
  if (tx == TX && ty == TY) {                                                          \
    auto k = plane_inv_fixed<Epi, TX, TY, T>;                                          \
    set_smem(k, p.smem_plane);                                                         \
    k<<<nitems, T, p.smem_plane, s>>>(tiles, items, pt.device(), spec, e, boxes);      \
    return true;                                                                       \
  }
  MVD_FIXED_PLANE_SHAPES(MVD_INV_CASE)
#undef MVD_INV_CASE
  return false;
}

template <class Epi>
static void launch_inv_impl(PlanTable& pt, const ConvPlan& p, const float2* spec, Epi e, cudaStream_t s) {
  if (p.items_inv.empty()) return;
  const int nitems = (int)p.items_inv.size();
  if (!launch_inv_fixed(pt, p, p.d_tiles.as<TileDesc>(), p.d_items_inv.as<int2>(), nitems, spec, e, s)) {
    auto k = plane_inv_kernel<Epi>;
    set_smem(k, p.smem_plane);
    const int threads = p.threads_plane > 0 ? p.threads_plane : kThreads;
    k<<<nitems, threads, p.smem_plane, s>>>(p.d_tiles.as<TileDesc>(), p.d_items_inv.as<int2>(), pt.device(), spec,
                                            e, epilogue_boxes(p, e));
  }
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

void launch_inv_store(PlanTable& pt, const ConvPlan& p, const float2* spec, float* out, cudaStream_t s) {
  EpiStore e{out, p.vol[0], p.vol[1]};
  launch_inv_impl(pt, p, spec, e, s);
}

void launch_inv_quotient(PlanTable& pt, const ConvPlan& p, const float2* spec, const float* img, float* q,
                         cudaStream_t s) {
  EpiQuotient e{img, q, p.vol[0], p.vol[1]};
  launch_inv_impl(pt, p, spec, e, s);
}

void launch_inv_update(PlanTable& pt, const ConvPlan& p, const float2* spec, float* psi, const float* weight,
                       float lambda, double* stat_sum, unsigned* stat_max, const StatArchive& archive,
                       cudaStream_t s) {
  EpiUpdate e{psi, weight, lambda, stat_sum, stat_max, p.vol[0], p.vol[1], 0.f, 0.f, archive};
  launch_inv_impl(pt, p, spec, e, s);
}

void launch_inv_nll(PlanTable& pt, const ConvPlan& p, const float2* spec, const float* img, const float* w, float* r,
                    double* nll, cudaStream_t s) {
  EpiNll e{img, w, r, nll, p.vol[0], p.vol[1], 0.f};
  launch_inv_impl(pt, p, spec, e, s);
}

void launch_inv_store_items(PlanTable& pt, const ConvPlan& p, const TileDesc* tiles, const int2* items, int nitems,
                            const float2* spec, float* out, int nx, int ny, cudaStream_t s) {
  if (nitems == 0) return;
  if (!launch_inv_fixed(pt, p, tiles, items, nitems, spec, EpiStore{out, nx, ny}, s)) {
    auto k = plane_inv_kernel<EpiStore>;
    set_smem(k, p.smem_plane);
    k<<<nitems, p.threads_plane > 0 ? p.threads_plane : kThreads, p.smem_plane, s>>>(tiles, items, pt.device(), spec,
                                                                                     EpiStore{out, nx, ny}, EpiBoxes{});
  }
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

}  // namespace mvd
