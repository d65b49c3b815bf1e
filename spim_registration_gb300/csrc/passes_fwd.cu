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

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to the driver library)
EncodeTiled encode_tiled() {
  static EncodeTiled fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return static_cast<EncodeTiled>(nullptr);
    return reinterpret_cast<EncodeTiled>(p);
  }();
  return fn;
}

// The slice-copy forward kernel is opt-in (MVD_TMA=1): with one slice per CTA the copy's latency
// stands in front of all of the CTA's work, and on cfg2 it measured slower (0.735 vs 0.62 ms of
// forward passes per iteration) than the gather that keeps ~20 loads per thread in flight.
bool use_tma() {
  static bool on = [] {
    const char* e = std::getenv("MVD_TMA");
    return e && e[0] == '1';
  }();
  return on;
}

// Tensor map of a float volume [nz][ny][nx] with a (w, h, 1) box; false when the volume does not
// meet the copy's rules (16-byte aligned base and row stride) or the driver refuses it.
bool volume_box_map(const float* base, int nx, int ny, int nz, int w, int h, CUtensorMap* out) {
  static std::mutex mu;
  static std::map<std::tuple<const float*, int, int, int, int, int>, CUtensorMap> cache;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (nx % 4) || w > 256 || h > 256) return false;
  const auto key = std::make_tuple(base, nx, ny, nz, w, h);
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(key);
  if (it != cache.end()) {
    *out = it->second;
    return true;
  }
  EncodeTiled enc = encode_tiled();
  if (!enc) return false;
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[2] = {(cuuint64_t)nx * sizeof(float), (cuuint64_t)nx * ny * sizeof(float)};
  const cuuint32_t box[3] = {(cuuint32_t)w, (cuuint32_t)h, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  if (enc(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  cache[key] = m;
  *out = m;
  return true;
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
  int n = 0;
  MVD_CHECK(cudaMemcpy(&n, tma_timeout_counter(), sizeof(int), cudaMemcpyDeviceToHost));
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
      auto k = plane_fwd_fixed<Gather, TX, TY, kFixedThreads>;                                            \
      set_smem(k, smem);                                                                                  \
      k<<<nitems, kFixedThreads, smem, s>>>(tiles, items, pt.device(), spec, g);                          \
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
    auto k = plane_fwd_kernel<Gather, MASK>;
    set_smem(k, smem);
    k<<<nitems, threads > 0 ? threads : kThreads, smem, s>>>(tiles, items, pt.device(), spec, g);
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
