// Host engine of the tiled FFT convolution: plans, tile planner, OTF preparation, launches,
// and the small elementwise / reduction kernels of the deconvolution path.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <cstdint>
#include <map>
#include <mutex>
#include <tuple>
#include <sstream>

#include "engine.h"

namespace mvd {

static std::atomic<long long> g_launches{0};
long long launch_count() { return g_launches.load(); }
void count_launch(int n) { g_launches += n; }

void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    throw CudaError(e, msg);
  }
}

namespace {
thread_local cudaStream_t tls_alloc_stream = nullptr;
}

AllocScope::AllocScope(cudaStream_t s) : prev_(tls_alloc_stream) { tls_alloc_stream = s; }
AllocScope::~AllocScope() { tls_alloc_stream = prev_; }
cudaStream_t alloc_stream() { return tls_alloc_stream; }

void upload_table(void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return;
  if (tls_alloc_stream)  // pageable source: staged before the call returns
    MVD_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, tls_alloc_stream));
  else
    MVD_CHECK(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
}

void keep_pool_memory(int dev) {
  static std::mutex mu;
  static std::vector<bool> done;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)done.size() <= dev) done.resize(dev + 1, false);
  if (done[dev]) return;
  cudaMemPool_t pool;
  MVD_CHECK(cudaDeviceGetDefaultMemPool(&pool, dev));
  uint64_t threshold = UINT64_MAX;
  MVD_CHECK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold));
  done[dev] = true;
}

void DevBuf::release() {
  if (p) {
    if (stream)
      cudaFreeAsync(p, stream);
    else
      cudaFree(p);
  }
  p = nullptr;
  bytes = 0;
  stream = nullptr;
}
DevBuf::~DevBuf() { release(); }
DevBuf& DevBuf::operator=(DevBuf&& o) noexcept {
  if (this != &o) {
    release();
    p = o.p;
    bytes = o.bytes;
    stream = o.stream;
    o.p = nullptr;
    o.bytes = 0;
    o.stream = nullptr;
  }
  return *this;
}
void DevBuf::alloc(size_t b) {
  release();
  if (b == 0) return;
  if (tls_alloc_stream) {
    MVD_CHECK(cudaMallocAsync(&p, b, tls_alloc_stream));
    stream = tls_alloc_stream;
  } else {
    MVD_CHECK(cudaMalloc(&p, b));
  }
  bytes = b;
}
void DevBuf::ensure(size_t b) {
  if (b > bytes) alloc(b);
}

bool is_smooth(int n) {
  if (n <= 0) return false;
  for (int f : {2, 3, 5})
    while (n % f == 0) n /= f;
  return n == 1;
}

int next_smooth(int n, bool even) {
  if (n < 2) n = 2;
  for (int m = n;; ++m) {
    if (even && (m & 1)) continue;
    if (is_smooth(m)) return m;
  }
}

// Radices of the register DFTs (fft_device.cuh).
static const int kRadices[] = {20, 18, 16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2};

static void best_split(int n, int depth, int maxdepth, std::vector<int>& cur, std::vector<int>& best) {
  if (n == 1) {
    // fewest stages first, then the most balanced (largest smallest radix)
    auto mn = [](const std::vector<int>& v) { return v.empty() ? 0 : *std::min_element(v.begin(), v.end()); };
    if (best.empty() || cur.size() < best.size() || (cur.size() == best.size() && mn(cur) > mn(best))) best = cur;
    return;
  }
  if (depth == maxdepth) return;
  for (int r : kRadices) {
    if (n % r) continue;
    if (!cur.empty() && r > cur.back()) continue;  // non-increasing order
    cur.push_back(r);
    best_split(n / r, depth + 1, maxdepth, cur, best);
    cur.pop_back();
  }
}

std::vector<int> factorize(int n) {
  if (n == 1) return {1};
  std::vector<int> cur, best;
  for (int depth = 1; depth <= kMaxStages && best.empty(); ++depth) best_split(n, 0, depth, cur, best);
  if (best.empty()) throw std::invalid_argument("FFT length is not 2,3,5-smooth");
  return best;
}

// ------------------------------------------------------------------------------------------
// plan table
// ------------------------------------------------------------------------------------------
int PlanTable::index_of(int n, bool ascending) {
  const int key = ascending ? -n : n;
  auto it = by_len_.find(key);
  if (it != by_len_.end()) return it->second;
  if (n < 1) throw std::invalid_argument("bad FFT length");
  if ((int)host_.size() >= kCapacity) throw std::runtime_error("FFT plan table full");
  FftPlan p{};
  p.n = n;
  std::vector<int> rad = factorize(n);
  if (ascending) std::reverse(rad.begin(), rad.end());
  if ((int)rad.size() > kMaxStages) throw std::invalid_argument("too many FFT stages");
  p.nstages = (int)rad.size();
  for (size_t i = 0; i < rad.size(); ++i) p.radix[i] = rad[i];
  // twiddles: [0, n) for the complex length n, then [0, n] for the real length 2n
  std::vector<float2> tw(2 * n + 1);
  for (int k = 0; k < n; ++k) {
    const double a = -2.0 * M_PI * (double)k / (double)n;
    tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  for (int k = 0; k <= n; ++k) {
    const double a = -M_PI * (double)k / (double)n;
    tw[n + k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  auto buf = std::make_unique<DevBuf>(tw.size() * sizeof(float2));
  upload_table(buf->p, tw.data(), tw.size() * sizeof(float2));
  p.tw = buf->as<float2>();
  p.tw_r2c = buf->as<float2>() + n;
  tw_bufs_.push_back(std::move(buf));
  const int idx = (int)host_.size();
  host_.push_back(p);
  by_len_[key] = idx;
  dirty_ = true;
  return idx;
}

const FftPlan* PlanTable::device() {
  if (!dev_.p) dev_.alloc(kCapacity * sizeof(FftPlan));
  if (dirty_) {
    // append-only table at a fixed address: entries already in use never change, so kernels
    // (and captured graphs) holding this pointer stay valid while new lengths are added
    upload_table(dev_.p, host_.data(), host_.size() * sizeof(FftPlan));
    dirty_ = false;
  }
  return dev_.as<FftPlan>();
}

// ------------------------------------------------------------------------------------------
// tile planner
// ------------------------------------------------------------------------------------------
static std::vector<AxisTiles> axis_options(int size, int k, bool even, int tmax) {
  std::vector<AxisTiles> out;
  int last_T = -1;
  const int nmax = std::max(1, size);
  for (int n = 1; n <= nmax && n <= 64; ++n) {
    const int need = (size + n - 1) / n + k - 1;
    int T = next_smooth(std::max(need, k), even);
    if (T > tmax) continue;
    if (T == last_T) continue;
    last_T = T;
    AxisTiles a;
    a.size = size;
    a.k = k;
    a.T = T;
    a.E = T - k + 1;
    a.n = (size + a.E - 1) / a.E;
    out.push_back(a);
    if (a.E < 8 && a.E < size) break;  // smaller tiles would be nearly all halo
  }
  return out;
}

// Work items of the three passes.  Plane passes: slice by slice, every tile of a slice before
// the next slice.  The forward pass then reads the halo a tile shares with its neighbours (30
// columns or rows of the 512x512x256 workload's 160-wide tiles) from L2 while the neighbours
// gather it, and the inverse pass's epilogue reads and writes each volume row, which the tiles
// of a slice split between them, within a short time (512x512x256 workload, per iteration:
// forward passes 2.91 against 2.99 ms, inverse passes 3.46 against 3.62 ms tile by tile).
// z pass: blocks
// of kZBlock consecutive pencil chunks, each block swept over every tile before the next.  All
// tiles of a plan share one kernel spectrum (the OTF), so a block's OTF chunks stay in L2 while
// every tile reads them, and each tile's reads stay contiguous over the block.  (Tile by tile,
// a view's OTF of up to 33 MB was re-read from DRAM for every tile; chunk by chunk across tiles,
// consecutive CTAs read 16 tiles' scattered chunks and the z pass got slower: 3.62 ms against
// 3.43 ms per iteration on the 512x512x256 workload.)
constexpr int kZBlock = 32;
static void fill_items(ConvPlan& p) {
  p.items_fwd.clear();
  p.items_inv.clear();
  p.items_z.clear();
  int plane_max = 0, tz_max = 0;
  for (int i = 0; i < (int)p.tiles.size(); ++i) {
    plane_max = std::max(plane_max, p.tiles[i].ty * p.tiles[i].px);
    tz_max = std::max(tz_max, p.tiles[i].tz);
  }
  for (int z = 0; z < tz_max; ++z)
    for (int i = 0; i < (int)p.tiles.size(); ++i) {
      const TileDesc& t = p.tiles[i];
      if (z >= t.hz && z < t.hz + t.ez) p.items_inv.push_back(make_int2(i, z));
    }
  for (int z = 0; z < tz_max; ++z)
    for (int i = 0; i < (int)p.tiles.size(); ++i)
      if (z < p.tiles[i].tz) p.items_fwd.push_back(make_int2(i, z));
  auto zitems = [&](std::vector<int2>& out, int chunk) {
    out.clear();
    for (int b0 = 0; b0 < plane_max; b0 += kZBlock * kZChunk)
      for (int i = 0; i < (int)p.tiles.size(); ++i) {
        const int plane = p.tiles[i].ty * p.tiles[i].px;
        for (int p0 = b0; p0 < std::min(plane, b0 + kZBlock * kZChunk); p0 += chunk)
          out.push_back(make_int2(i, p0));
      }
  };
  zitems(p.items_z, kZChunk);
  zitems(p.items_zw, kZWideChunk);
}

void ConvPlan::upload() {
  d_tiles.alloc(tiles.size() * sizeof(TileDesc));
  upload_table(d_tiles.p, tiles.data(), tiles.size() * sizeof(TileDesc));
  auto up = [](DevBuf& b, const std::vector<int2>& v) {
    b.alloc(std::max<size_t>(1, v.size()) * sizeof(int2));
    if (!v.empty()) upload_table(b.p, v.data(), v.size() * sizeof(int2));
  };
  up(d_items_fwd, items_fwd);
  up(d_items_inv, items_inv);
  up(d_items_z, items_z);
  up(d_items_zw, items_zw);
  // OTF build tables: one tile of this shape covering [0, T) with its full region effective
  if (!tiles.empty()) {
    TileDesc t = tiles[0];
    t.ox = t.oy = t.oz = 0;
    t.hx = t.hy = t.hz = 0;
    t.ex = t.tx; t.ey = t.ty; t.ez = t.tz;
    t.spec_off = 0;
    t.otf_off = 0;
    std::vector<int2> fwd, zz;
    for (int z = 0; z < t.tz; ++z) fwd.push_back(make_int2(0, z));
    for (int p0 = 0; p0 < t.ty * t.px; p0 += kZChunk) zz.push_back(make_int2(0, p0));
    d_otf_tile.alloc(sizeof(TileDesc));
    upload_table(d_otf_tile.p, &t, sizeof(TileDesc));
    up(d_otf_fwd, fwd);
    up(d_otf_z, zz);
    n_otf_fwd = (int)fwd.size();
    n_otf_z = (int)zz.size();
  }
}

// Shared-memory budget of one plane buffer used by the planner (MVD_PLANE_CAP overrides it;
// planes of at most half the budget let two CTAs share an SM).
int plane_cap() {
  static int cap = [] {
    const char* e = std::getenv("MVD_PLANE_CAP");
    int v = e ? std::atoi(e) : 0;
    return (v >= 256 && v <= kPlaneCap) ? v : kPlaneCapDefault;
  }();
  return cap;
}

static bool plane_cap_from_env() {
  const char* e = std::getenv("MVD_PLANE_CAP");
  const int v = e ? std::atoi(e) : 0;
  return v >= 256 && v <= kPlaneCap;
}

int plane_limit() { return plane_cap_from_env() ? plane_cap() : kPlaneCap; }

double plane_cost_factor(int tx, int ty, long long plane) {
  if (plane_cap_from_env()) return 1.0;
  const bool two_per_sm = plane <= kPlaneCapDefault || (use_staged_planes() && staged_plane_shape(tx, ty));
  double f = two_per_sm ? 1.0 : 1.12;
  if (!compiled_plane_shape(tx, ty)) f *= 1.3;
  return f;
}

int plane_threads() {
  static int t = [] {
    const char* e = std::getenv("MVD_PLANE_THREADS");
    int v = e ? std::atoi(e) : 0;
    return (v >= 64 && v <= kThreads && v % 32 == 0) ? v : kThreads;
  }();
  return t;
}

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

}  // namespace

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
  if (cache.size() >= 4096) cache.clear();  // maps are cheap to encode again; bound the memory
  cache[key] = m;
  *out = m;
  return true;
}


bool use_l2_prefetch() {
  static bool on = [] {
    const char* e = std::getenv("MVD_L2_PREFETCH");
    return !(e && e[0] == '0');
  }();
  return on;
}

bool use_staged_planes() {
  static bool on = [] {
    const char* e = std::getenv("MVD_STAGED_PLANES");
    return !(e && e[0] == '0');
  }();
  return on;
}

bool use_fixed_planes() {
  static bool on = [] {
    const char* e = std::getenv("MVD_FIXED_PLANES");
    return !(e && e[0] == '0');
  }();
  return on;
}

std::unique_ptr<ConvPlan> make_conv_plan(PlanTable& pt, int nx, int ny, int nz, int kx, int ky,
                                         int kz, const PlanOptions& opt) {
  if (nx < 1 || ny < 1 || nz < 1) throw std::invalid_argument("empty volume");
  if (kx < 1 || ky < 1 || kz < 1 || !(kx & 1) || !(ky & 1) || !(kz & 1))
    throw std::invalid_argument("kernel sizes must be odd and positive");
  auto opts = [&](int size, int k, bool even, int tmax, int force) {
    if (force > 0) {
      AxisTiles a;
      a.size = size;
      a.k = k;
      a.T = force;
      a.E = force - k + 1;
      if (a.E <= 0 || (even && (force & 1)) || !is_smooth(even ? force / 2 : force))
        throw std::invalid_argument("forced tile size is too small or not smooth");
      a.n = (size + a.E - 1) / a.E;
      return std::vector<AxisTiles>{a};
    }
    return axis_options(size, k, even, tmax);
  };
  auto ox = opts(nx, kx, true, 2 * (kPlaneCap / 8), opt.force_tx);
  auto oy = opts(ny, ky, false, kPlaneCap / 2, opt.force_ty);
  auto oz = opts(nz, kz, false, kPlaneCap / kZPitch, opt.force_tz);
  double best = 1e300;
  AxisTiles bx, by, bz;
  // an explicit budget (the autotuner's candidates) is a hard limit; the default plan weighs
  // the plane size and the compiled shapes (plane_cost_factor)
  const int limit = opt.cap > 0 ? opt.cap : plane_limit();
  for (auto& a : ox)
    for (auto& b : oy) {
      const long long plane = (long long)row_pitch(a.T / 2) * b.T;
      if (plane > limit) continue;
      const double factor = opt.cap > 0 ? 1.0 : plane_cost_factor(a.T, b.T, plane);
      for (auto& c : oz) {
        const double ntiles = (double)a.n * b.n * c.n;
        const double cost = ntiles * a.T * b.T * c.T * (1.0 + 1e-3 * ntiles) * factor;
        if (cost < best) {
          best = cost;
          bx = a;
          by = b;
          bz = c;
        }
      }
    }
  if (best >= 1e300) throw std::invalid_argument("no tile shape fits this kernel (kernel too large)");
  auto plan = std::make_unique<ConvPlan>();
  ConvPlan& p = *plan;
  p.nx = nx; p.ny = ny; p.nz = nz;
  p.kx = kx; p.ky = ky; p.kz = kz;
  p.vol[0] = nx; p.vol[1] = ny; p.vol[2] = nz;
  p.box_hi[0] = nx; p.box_hi[1] = ny; p.box_hi[2] = nz;
  p.ax = bx; p.ay = by; p.az = bz;
  const int px = bx.T / 2 + 1;
  const int pitch = row_pitch(bx.T / 2);
  const int plx = pt.index_of(bx.T / 2, opt.ascending), ply = pt.index_of(by.T, opt.ascending),
            plz = pt.index_of(bz.T, opt.ascending);
  const long long tile_spec = (long long)px * by.T * bz.T;
  long long off = 0;
  for (int iz = 0; iz < bz.n; ++iz)
    for (int iy = 0; iy < by.n; ++iy)
      for (int ix = 0; ix < bx.n; ++ix) {
        TileDesc t{};
        t.tx = bx.T; t.ty = by.T; t.tz = bz.T;
        t.px = px;
        t.pitch = pitch;
        t.hx = kx / 2; t.hy = ky / 2; t.hz = kz / 2;
        const int ex0 = ix * bx.E, ey0 = iy * by.E, ez0 = iz * bz.E;
        t.ox = ex0 - kx / 2; t.oy = ey0 - ky / 2; t.oz = ez0 - kz / 2;
        t.ex = std::min(bx.E, nx - ex0);
        t.ey = std::min(by.E, ny - ey0);
        t.ez = std::min(bz.E, nz - ez0);
        t.plan_x = plx; t.plan_y = ply; t.plan_z = plz;
        t.spec_off = off;
        t.otf_off = 0;
        off += tile_spec;
        p.tiles.push_back(t);
      }
  p.spec_elems = off;
  p.otf_elems = tile_spec;
  p.smem_plane = 2 * (size_t)by.T * pitch * sizeof(float2);
  p.threads_plane = opt.threads > 0 ? opt.threads : plane_threads();
  p.ascending = opt.ascending;
  p.generic = opt.generic || opt.ascending;  // compiled kernels hold the descending order
  p.staged = use_staged_planes();
  p.smem_z = 2 * (size_t)bz.T * kZPitch * sizeof(float2);
  fill_items(p);
  p.upload();
  return plan;
}

void place_plan(ConvPlan& p, int dx, int dy, int dz, const int vol[3]) {
  for (auto& t : p.tiles) {
    t.ox += dx;
    t.oy += dy;
    t.oz += dz;
  }
  const int d[3] = {dx, dy, dz}, n[3] = {p.nx, p.ny, p.nz};
  for (int i = 0; i < 3; ++i) {
    p.vol[i] = vol[i];
    p.box_lo[i] = d[i];
    p.box_hi[i] = d[i] + n[i];
  }
  p.upload();
}

std::string describe(const ConvPlan& p) {
  std::ostringstream os;
  os << "volume " << p.nx << "x" << p.ny << "x" << p.nz << " kernel " << p.kx << "x" << p.ky << "x"
     << p.kz << " tiles " << p.ax.n << "x" << p.ay.n << "x" << p.az.n << " of " << p.ax.T << "x"
     << p.ay.T << "x" << p.az.T << " (effective " << p.ax.E << "x" << p.ay.E << "x" << p.az.E
     << "), padded/volume " << (double)p.padded_voxels() / ((double)p.nx * p.ny * p.nz);
  return os.str();
}

// ------------------------------------------------------------------------------------------
// launches (the pass kernels are instantiated in passes_fwd.cu, passes_inv.cu, passes_z.cu)
// ------------------------------------------------------------------------------------------
// raise a kernel's dynamic shared-memory limit once per (device, kernel, size)
void set_smem_raw(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> done;
  int dev = 0;
  MVD_CHECK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(dev, kernel);
  auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return;
  MVD_CHECK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  done[key] = bytes;
}

void convolve(PlanTable& pt, const ConvPlan& plan, const float* in, Ext ext, float value,
              const float2* otf, float2* spec, float* out, cudaStream_t s) {
  if (ext == Ext::Mirror)
    launch_fwd_mirror(pt, plan, in, spec, s);
  else
    launch_fwd_value(pt, plan, in, value, spec, s);
  launch_z(pt, plan, spec, otf, s);
  launch_inv_store(pt, plan, spec, out, s);
}

// ------------------------------------------------------------------------------------------
// OTF: kernel placed with its centre at the tile origin (wrap-around), forward 3D FFT,
// scaled by 1 / (tx ty tz) so that the unnormalised inverse transforms give the convolution.
// ------------------------------------------------------------------------------------------
__global__ void place_kernel_kernel(const float* __restrict__ k, int kx, int ky, int kz, float* __restrict__ vol,
                                    int tx, int ty, int tz) {
  const long long n = (long long)kx * ky * kz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % kx);
    const int y = (int)((i / kx) % ky);
    const int z = (int)(i / ((long long)kx * ky));
    const int wx = ((x - kx / 2) % tx + tx) % tx;
    const int wy = ((y - ky / 2) % ty + ty) % ty;
    const int wz = ((z - kz / 2) % tz + tz) % tz;
    vol[((long long)wz * ty + wy) * tx + wx] = k[i];
  }
}

void build_otf(PlanTable& pt, const ConvPlan& plan, const float* kernel, float2* otf, DevBuf& scratch,
               cudaStream_t s) {
  const int tx = plan.ax.T, ty = plan.ay.T, tz = plan.az.T;
  if (plan.kx > tx || plan.ky > ty || plan.kz > tz) throw std::invalid_argument("kernel larger than tile");
  const size_t vox = (size_t)tx * ty * tz;
  scratch.ensure(vox * sizeof(float));
  MVD_CHECK(cudaMemsetAsync(scratch.p, 0, vox * sizeof(float), s));
  const long long kn = (long long)plan.kx * plan.ky * plan.kz;
  place_kernel_kernel<<<(int)std::min<long long>((kn + 255) / 256, 4096), 256, 0, s>>>(
      kernel, plan.kx, plan.ky, plan.kz, scratch.as<float>(), tx, ty, tz);
  MVD_CHECK(cudaGetLastError());
  count_launch();
  // one tile covering the placed kernel volume exactly; its spectrum goes to `otf`
  launch_fwd_value_items(pt, plan, plan.d_otf_tile.as<TileDesc>(), plan.d_otf_fwd.as<int2>(), plan.n_otf_fwd,
                         scratch.as<float>(), tx, ty, tz, 0.f, otf, s);
  launch_z_forward_scaled(pt, plan, plan.d_otf_tile.as<TileDesc>(), plan.d_otf_z.as<int2>(), plan.n_otf_z, otf,
                          (float)(1.0 / ((double)tx * ty * tz)), s);
}

// ------------------------------------------------------------------------------------------
// elementwise and reduction kernels
// ------------------------------------------------------------------------------------------
static int grid_for(long long n, int threads = 256) {
  long long b = (n + threads - 1) / threads;
  return (int)std::max<long long>(1, std::min<long long>(b, 152LL * 16));
}

__device__ __forceinline__ void block_reduce_add2(double a, double b, double* out) {
  __shared__ double ra[32], rb[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { ra[warp] = a; rb[warp] = b; }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    a = lane < nw ? ra[lane] : 0.0;
    b = lane < nw ? rb[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
      atomicAdd(out, a);
      atomicAdd(out + 1, b);
    }
  }
}

__global__ void sum_f64_kernel(const float* __restrict__ x, long long n, double* out) {
  double a = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a += (double)x[i];
  __shared__ double r[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) r[warp] = a;
  __syncthreads();
  if (warp == 0) {
    a = lane < (int)(blockDim.x >> 5) ? r[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) atomicAdd(out, a);
  }
}

void dev_sum_f64(const float* x, long long n, double* out, cudaStream_t s) {
  sum_f64_kernel<<<grid_for(n), 256, 0, s>>>(x, n, out);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

__global__ void scale_div_kernel(float* x, long long n, const double* d) {
  const double div = *d;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = (float)((double)x[i] / div);
}

void dev_scale_div(float* x, long long n, const double* d, cudaStream_t s) {
  scale_div_kernel<<<grid_for(n), 256, 0, s>>>(x, n, d);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

// Mirror.mirror along every axis: p <-> n-1-p for p <= n/2 (for even n the middle pair is
// swapped twice and stays in place: Mirror.java:94-112)
__device__ __forceinline__ int mirror_pos(int p, int n) {
  if ((n & 1) == 0 && (p == n / 2 - 1 || p == n / 2)) return p;
  return n - 1 - p;
}

__global__ void mirror_kernel(const float* __restrict__ in, float* __restrict__ out, int nx, int ny, int nz) {
  const long long n = (long long)nx * ny * nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx);
    const int y = (int)((i / nx) % ny);
    const int z = (int)(i / ((long long)nx * ny));
    out[i] = in[((long long)mirror_pos(z, nz) * ny + mirror_pos(y, ny)) * nx + mirror_pos(x, nx)];
  }
}

void dev_mirror(const float* in, float* out, int nx, int ny, int nz, cudaStream_t s) {
  mirror_kernel<<<grid_for((long long)nx * ny * nz), 256, 0, s>>>(in, out, nx, ny, nz);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

__global__ void mul_kernel(float* a, const float* b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = __fmul_rn(a[i], b[i]);
}
void dev_mul(float* a, const float* b, long long n, cudaStream_t s) {
  mul_kernel<<<grid_for(n), 256, 0, s>>>(a, b, n);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

// MVDeconFFT.pow (:346-354): repeated float multiplication
__global__ void pow_kernel(float* a, int power, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float v = a[i];
    float r = v;
    for (int k = 1; k < power; ++k) r = __fmul_rn(r, v);
    a[i] = r;
  }
}
void dev_pow(float* a, int power, long long n, cudaStream_t s) {
  pow_kernel<<<grid_for(n), 256, 0, s>>>(a, power, n);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

__global__ void fill_kernel(float* a, float v, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = v;
}
void dev_fill(float* a, float v, long long n, cudaStream_t s) {
  fill_kernel<<<grid_for(n), 256, 0, s>>>(a, v, n);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

struct ViewPtrs {
  const float* p[16];
};

// FirstIteration.call (FirstIteration.java:84-154): per voxel the mean of the positive view
// values; summed (FP64) over voxels with at least one positive value, and counted.
// hi + lo = a + b exactly (Knuth's two-sum)
__device__ __forceinline__ void two_sum(float a, float b, float& hi, float& lo) {
  hi = __fadd_rn(a, b);
  const float bb = __fsub_rn(hi, a);
  lo = __fadd_rn(__fsub_rn(a, __fsub_rn(hi, bb)), __fsub_rn(b, bb));
}

// (hi, lo) += (bh, bl), renormalised; ~2^-44 relative
__device__ __forceinline__ void pair_add(float& hi, float& lo, float bh, float bl) {
  float s, e;
  two_sum(hi, bh, s, e);
  e = __fadd_rn(e, __fadd_rn(lo, bl));
  hi = __fadd_rn(s, e);
  lo = __fsub_rn(e, __fsub_rn(hi, s));
}

// FirstIteration.compatibleLoop (FirstIteration.java:124-154): per voxel the mean of the
// views' positive values, summed over the voxels that have any (RealSum), and their count.
// GB300's FP64 pipe cannot take a double division and six double additions per voxel at
// HBM speed, so each thread carries its sum as a float pair (the voxel's view sum by exact
// two-sums, times 1/c as a pair), flushed into a double every 16 voxels.  The reference's
// RealSum is itself order-dependent; each pair chunk is accurate to ~2^-43.
__global__ void first_iteration_kernel(ViewPtrs v, int nviews, long long n, double* out) {
  float acc_hi = 0.f, acc_lo = 0.f;
  double total = 0.0;
  unsigned long long cnt = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float s_hi = 0.f, s_lo = 0.f;
    int c = 0;
    for (int k = 0; k < nviews; ++k) {
      const float x = __ldg(v.p[k] + i);
      if (x > 0.f) {
        float e;
        two_sum(s_hi, x, s_hi, e);
        s_lo = __fadd_rn(s_lo, e);
        ++c;
      }
    }
    if (c > 0) {
      // (s_hi + s_lo) / c: q = s_hi / c rounded, the remainder s_hi - q c is exact (an FMA)
      const float fc = (float)c;
      const float q = __fdiv_rn(s_hi, fc);
      const float r = __fadd_rn(__fmaf_rn(-q, fc, s_hi), s_lo);
      pair_add(acc_hi, acc_lo, q, __fdiv_rn(r, fc));
      if ((++cnt & 15) == 0) {
        total += (double)acc_hi + (double)acc_lo;
        acc_hi = acc_lo = 0.f;
      }
    }
  }
  block_reduce_add2(total + ((double)acc_hi + (double)acc_lo), (double)cnt, out);
}

void dev_first_iteration(const float* const* views, int nviews, long long n, double* out, cudaStream_t s) {
  ViewPtrs vp{};
  if (nviews > 16) throw std::invalid_argument("at most 16 views");
  for (int i = 0; i < nviews; ++i) vp.p[i] = views[i];
  first_iteration_kernel<<<grid_for(n), 256, 0, s>>>(vp, nviews, n, out);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

// MVDeconvolution.java:133-147: psi := avg (0.5 if NaN)
__global__ void fill_avg_kernel(float* psi, const double* sc, long long n) {
  double avg = sc[0] / sc[1];
  if (isnan(avg)) avg = 0.5;
  const float v = (float)avg;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    psi[i] = v;
}
void dev_fill_from_avg(float* psi, const double* sc, long long n, cudaStream_t s) {
  fill_avg_kernel<<<grid_for(n), 256, 0, s>>>(psi, sc, n);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

// MVDeconvolution.java:201-208: psi := 0 where no view has data
__global__ void mask_kernel(float* psi, ViewPtrs v, int nviews, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    bool any = false;
    for (int k = 0; k < nviews; ++k) any |= __ldg(v.p[k] + i) > 0.f;
    if (!any) psi[i] = 0.f;
  }
}
void dev_mask(float* psi, const float* const* views, int nviews, long long n, cudaStream_t s) {
  ViewPtrs vp{};
  if (nviews > 16) throw std::invalid_argument("at most 16 views");
  for (int i = 0; i < nviews; ++i) vp.p[i] = views[i];
  mask_kernel<<<grid_for(n), 256, 0, s>>>(psi, vp, nviews, n);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

__global__ void quotient_kernel(float* b, const float* img, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float x = img[i];
    b[i] = EpiQuotient::quotient(x, b[i]);
  }
}
void dev_quotient(float* b, const float* img, long long n, cudaStream_t s) {
  quotient_kernel<<<grid_for(n), 256, 0, s>>>(b, img, n);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

__global__ void update_kernel(float* psi, const float* integral, const float* weight, float lambda, long long n,
                              double* stat_sum, unsigned* stat_max) {
  EpiUpdate e{psi, weight, lambda, stat_sum, stat_max, 0, 0, 0.f, 0.f, StatArchive{}};
  e.acc_init();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    e(i, integral[i]);
  e.finish();
}
void dev_update(float* psi, const float* integral, const float* weight, float lambda, long long n,
                double* stat_sum, unsigned* stat_max, cudaStream_t s) {
  update_kernel<<<grid_for(n), 256, 0, s>>>(psi, integral, weight, lambda, n, stat_sum, stat_max);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

__global__ void copy_block_kernel(const float* __restrict__ vol, int nx, int ny, int nz, float* __restrict__ blk,
                                  int bx, int by, int bz, int ox, int oy, int oz, int mode, float value) {
  const long long n = (long long)bx * by * bz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % bx) + ox;
    const int y = (int)((i / bx) % by) + oy;
    const int z = (int)(i / ((long long)bx * by)) + oz;
    float v;
    if (mode == 0) {
      v = vol[((long long)mirror_single(z, nz) * ny + mirror_single(y, ny)) * nx + mirror_single(x, nx)];
    } else {
      v = (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) ? value
                                                                      : vol[((long long)z * ny + y) * nx + x];
    }
    blk[i] = v;
  }
}
void dev_copy_block(const float* vol, int nx, int ny, int nz, float* block, int bx, int by, int bz, int ox,
                    int oy, int oz, Ext ext, float value, cudaStream_t s) {
  copy_block_kernel<<<grid_for((long long)bx * by * bz), 256, 0, s>>>(vol, nx, ny, nz, block, bx, by, bz, ox, oy,
                                                                    oz, ext == Ext::Mirror ? 0 : 1, value);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

__global__ void paste_block_kernel(const float* __restrict__ blk, int bx, int by, int lx, int ly, int lz,
                                   float* __restrict__ vol, int nx, int ny, int ex0, int ey0, int ez0, int sx,
                                   int sy, int sz) {
  const long long n = (long long)sx * sy * sz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % sx);
    const int y = (int)((i / sx) % sy);
    const int z = (int)(i / ((long long)sx * sy));
    vol[((long long)(ez0 + z) * ny + (ey0 + y)) * nx + (ex0 + x)] =
        blk[((long long)(lz + z) * by + (ly + y)) * bx + (lx + x)];
  }
}
void dev_paste_block(const float* block, int bx, int by, int bz, int lx, int ly, int lz, float* vol, int nx,
                     int ny, int nz, int ex0, int ey0, int ez0, int sx, int sy, int sz, cudaStream_t s) {
  (void)bz;
  (void)nz;
  paste_block_kernel<<<grid_for((long long)sx * sy * sz), 256, 0, s>>>(block, bx, by, lx, ly, lz, vol, nx, ny, ex0,
                                                                     ey0, ez0, sx, sy, sz);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

__global__ void data_box_kernel(const float* __restrict__ img, const float* __restrict__ w, int nx, int ny, int nz,
                                int* box) {
  int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {-1, -1, -1};
  const long long n = (long long)nx * ny * nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (__ldg(img + i) > 0.f || __ldg(w + i) > 0.f) {
      const int c[3] = {(int)(i % nx), (int)((i / nx) % ny), (int)(i / ((long long)nx * ny))};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        lo[d] = min(lo[d], c[d]);
        hi[d] = max(hi[d], c[d]);
      }
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = min(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = max(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (hi[d] >= 0) {
        atomicMin(box + d, lo[d]);
        atomicMax(box + 3 + d, hi[d]);
      }
    }
  }
}

void dev_data_box(const float* img, const float* w, int nx, int ny, int nz, int* box, cudaStream_t s) {
  data_box_kernel<<<grid_for((long long)nx * ny * nz), 256, 0, s>>>(img, w, nx, ny, nz, box);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

}  // namespace mvd
