// mvd_convolve3d_device_noalloc: the device-pointer convolution without any device allocation.
//
// Who needs it: callers that are not allowed to call cudaMalloc / cudaFree while they run,
// for example an acquisition pipeline that deconvolves blocks while the microscope streams and
// must not take the device-wide synchronisation or the latency jitter of an allocation, or a
// host framework (a JVM plugin, an image server) whose own memory manager owns the device
// memory pool.  Every working buffer of this entry point -- FFT plans and twiddles, tile and
// work-item tables, the kernel's placed copy, its spectrum and the tile spectra -- is carved
// out of one file-scope __device__ array of fixed size, kScratchBytes, which every GPU that
// loads the library holds until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the array's device
// address with cudaGetSymbolAddress and keeps it.  Each call copies its plans and tables from
// host vectors that are freed on return, so a call on a stream that is being captured is
// refused.  A NULL stream is the legacy default stream, and the call returns once its work is
// enqueued.  Every call shares the array and its contents are whatever the last call left
// there, so calls whose GPU work overlaps (another stream, another host thread) race on it;
// callers serialise them.  The placed-kernel buffer is cleared on every call.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/mvdecon.h"
#include "engine.h"

using namespace mvd;

namespace mvd {
void set_last_error(const std::string& msg);  // capi.cu: the message mvd_last_error() returns
}

namespace {

constexpr size_t kScratchBytes = 64ull << 20;  // 64 MiB per device
constexpr int kMaxDevices = 64;

// The scratch memory.  In host code this name is only a host-side stand-in for the device
// array: kernels receive the address that cudaGetSymbolAddress returns.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {};

unsigned char* scratch_address(int dev) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) throw CudaError(e, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_addr[dev] = static_cast<unsigned char*>(p);
  }
  return g_addr[dev];
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct Axis {
  int T, n, E;
};

// tile choice: the allocating path's default rule (plane_limit, plane_cost_factor), so both
// pick the same tiles
std::vector<Axis> options(int size, int k, bool even, int tmax) {
  std::vector<Axis> out;
  int last = -1;
  for (int n = 1; n <= size && n <= 64; ++n) {
    const int need = (size + n - 1) / n + k - 1;
    const int T = next_smooth(need > k ? need : k, even);
    if (T > tmax || T == last) continue;
    last = T;
    const int E = T - k + 1;
    out.push_back({T, (size + E - 1) / E, E});
    if (E < 8 && E < size) break;
  }
  return out;
}

__global__ void place_kernel_noalloc(const float* __restrict__ k, int kx, int ky, int kz, float* __restrict__ vol,
                                     int tx, int ty, int tz) {
  const long long n = (long long)kx * ky * kz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % kx), y = (int)((i / kx) % ky), z = (int)(i / ((long long)kx * ky));
    const int wx = ((x - kx / 2) % tx + tx) % tx;
    const int wy = ((y - ky / 2) % ty + ty) % ty;
    const int wz = ((z - kz / 2) % tz + tz) % tz;
    vol[((long long)wz * ty + wy) * tx + wx] = k[i];
  }
}

}  // namespace

extern "C" int mvd_convolve3d_device_noalloc(const float* in, float* out, const int* dims, const float* kernel,
                                             const int* kd, int ext_mode, float ext_value, int devCUDA,
                                             void* stream) {
  try {
    set_last_error("");
    if (!in || !out || !kernel || !dims || !kd) {
      set_last_error("NULL pointer");
      return MVD_ERR_ARG;
    }
    for (int d = 0; d < 3; ++d) {
      if (dims[d] < 1 || kd[d] < 1) {
        set_last_error("sizes must be positive");
        return MVD_ERR_ARG;
      }
      if (!(kd[d] & 1)) {
        set_last_error("kernel sizes must be odd");
        return MVD_ERR_ARG;
      }
    }
    if (ext_mode != 0 && ext_mode != 1) {
      set_last_error("ext_mode must be 0 or 1");
      return MVD_ERR_ARG;
    }
    int count = 0;
    MVD_CHECK(cudaGetDeviceCount(&count));
    if (devCUDA < 0 || devCUDA >= count || devCUDA >= kMaxDevices) {
      set_last_error("invalid CUDA device id");
      return MVD_ERR_ARG;
    }
    MVD_CHECK(cudaSetDevice(devCUDA));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the tables below are copied from host vectors that are freed on return: a graph captured
    // from this call would read freed host memory, so a capturing stream is refused
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    MVD_CHECK(cudaStreamIsCapturing(s, &cap));
    if (cap != cudaStreamCaptureStatusNone) {
      set_last_error("mvd_convolve3d_device_noalloc cannot be called while its stream is being captured");
      return MVD_ERR_STATE;
    }
    unsigned char* base = scratch_address(devCUDA);

    // ---- tile plan (host only) ----
    const int nx = dims[0], ny = dims[1], nz = dims[2];
    auto ox = options(nx, kd[0], true, 2 * (kPlaneCap / 8));
    auto oy = options(ny, kd[1], false, kPlaneCap / 2);
    auto oz = options(nz, kd[2], false, kPlaneCap / kZPitch);
    double best = 1e300;
    Axis bx{}, by{}, bz{};
    for (auto& a : ox)
      for (auto& b : oy) {
        const long long plane = (long long)row_pitch(a.T / 2) * b.T;
        if (plane > plane_limit()) continue;
        const double factor = plane_cost_factor(a.T, b.T, plane);
        for (auto& c : oz) {
          const double nt = (double)a.n * b.n * c.n;
          const double cost = nt * a.T * b.T * c.T * (1.0 + 1e-3 * nt) * factor;
          if (cost < best) {
            best = cost;
            bx = a;
            by = b;
            bz = c;
          }
        }
      }
    if (best >= 1e300) {
      set_last_error("no tile shape fits this kernel");
      return MVD_ERR_ARG;
    }
    const int px = bx.T / 2 + 1;
    const int pitch = row_pitch(bx.T / 2);
    const int lens[3] = {bx.T / 2, by.T, bz.T};

    // FFT plans for the three lengths, twiddles computed in double on the host
    FftPlan plans[3];
    std::vector<std::vector<float2>> tws(3);
    for (int i = 0; i < 3; ++i) {
      const int n = lens[i];
      FftPlan p{};
      p.n = n;
      std::vector<int> rad = factorize(n);
      p.nstages = (int)rad.size();
      for (size_t r = 0; r < rad.size(); ++r) p.radix[r] = rad[r];
      plans[i] = p;
      auto& tw = tws[i];
      tw.resize(2 * n + 1);
      for (int k = 0; k < n; ++k) {
        const double a = -2.0 * M_PI * (double)k / (double)n;
        tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
      }
      for (int k = 0; k <= n; ++k) {
        const double a = -M_PI * (double)k / (double)n;
        tw[n + k] = make_float2((float)std::cos(a), (float)std::sin(a));
      }
    }

    // tiles and work items: tile 0 is the OTF tile, tiles 1.. cover the volume
    std::vector<TileDesc> tiles;
    TileDesc o{};
    o.tx = bx.T; o.ty = by.T; o.tz = bz.T;
    o.px = px; o.pitch = pitch;
    o.ex = bx.T; o.ey = by.T; o.ez = bz.T;
    o.plan_x = 0; o.plan_y = 1; o.plan_z = 2;
    tiles.push_back(o);
    const long long tile_spec = (long long)px * by.T * bz.T;
    long long off = 0;
    for (int iz = 0; iz < bz.n; ++iz)
      for (int iy = 0; iy < by.n; ++iy)
        for (int ix = 0; ix < bx.n; ++ix) {
          TileDesc t = o;
          t.hx = kd[0] / 2; t.hy = kd[1] / 2; t.hz = kd[2] / 2;
          const int ex0 = ix * bx.E, ey0 = iy * by.E, ez0 = iz * bz.E;
          t.ox = ex0 - kd[0] / 2; t.oy = ey0 - kd[1] / 2; t.oz = ez0 - kd[2] / 2;
          t.ex = std::min(bx.E, nx - ex0);
          t.ey = std::min(by.E, ny - ey0);
          t.ez = std::min(bz.E, nz - ez0);
          t.spec_off = off;
          t.otf_off = 0;
          off += tile_spec;
          tiles.push_back(t);
        }
    std::vector<int2> otf_fwd, otf_z, fwd, inv, zz;
    const int plane = by.T * px;
    for (int z = 0; z < bz.T; ++z) otf_fwd.push_back(make_int2(0, z));
    for (int p0 = 0; p0 < plane; p0 += kZChunk) otf_z.push_back(make_int2(0, p0));
    for (int i = 1; i < (int)tiles.size(); ++i) {
      for (int z = 0; z < bz.T; ++z) fwd.push_back(make_int2(i, z));
      for (int z = tiles[i].hz; z < tiles[i].hz + tiles[i].ez; ++z) inv.push_back(make_int2(i, z));
      for (int p0 = 0; p0 < plane; p0 += kZChunk) zz.push_back(make_int2(i, p0));
    }

    // ---- arena layout inside the static scratch ----
    size_t at = 0;
    auto take = [&](size_t bytes) {
      const size_t o2 = at;
      at = align256(at + bytes);
      return o2;
    };
    const size_t o_plans = take(sizeof(plans));
    size_t o_tw[3];
    for (int i = 0; i < 3; ++i) o_tw[i] = take(tws[i].size() * sizeof(float2));
    const size_t o_tiles = take(tiles.size() * sizeof(TileDesc));
    const size_t o_ofwd = take(otf_fwd.size() * sizeof(int2));
    const size_t o_oz = take(otf_z.size() * sizeof(int2));
    const size_t o_fwd = take(fwd.size() * sizeof(int2));
    const size_t o_inv = take(std::max<size_t>(1, inv.size()) * sizeof(int2));
    const size_t o_z = take(zz.size() * sizeof(int2));
    const size_t o_place = take((size_t)bx.T * by.T * bz.T * sizeof(float));
    const size_t o_otf = take((size_t)tile_spec * sizeof(float2));
    const size_t o_spec = take((size_t)off * sizeof(float2));
    if (at > kScratchBytes) {
      set_last_error("convolution needs " + std::to_string(at) + " bytes of scratch; the static scratch holds " +
                     std::to_string(kScratchBytes) + " bytes (use mvd_convolve3d_device for larger volumes)");
      return MVD_ERR_ARG;
    }
    for (int i = 0; i < 3; ++i) {
      plans[i].tw = reinterpret_cast<const float2*>(base + o_tw[i]);
      plans[i].tw_r2c = plans[i].tw + lens[i];
    }
    auto up = [&](size_t o3, const void* src, size_t bytes) {
      if (bytes) MVD_CHECK(cudaMemcpyAsync(base + o3, src, bytes, cudaMemcpyHostToDevice, s));
    };
    up(o_plans, plans, sizeof(plans));
    for (int i = 0; i < 3; ++i) up(o_tw[i], tws[i].data(), tws[i].size() * sizeof(float2));
    up(o_tiles, tiles.data(), tiles.size() * sizeof(TileDesc));
    up(o_ofwd, otf_fwd.data(), otf_fwd.size() * sizeof(int2));
    up(o_oz, otf_z.data(), otf_z.size() * sizeof(int2));
    up(o_fwd, fwd.data(), fwd.size() * sizeof(int2));
    up(o_inv, inv.data(), inv.size() * sizeof(int2));
    up(o_z, zz.data(), zz.size() * sizeof(int2));

    const FftPlan* d_plans = reinterpret_cast<const FftPlan*>(base + o_plans);
    const TileDesc* d_tiles = reinterpret_cast<const TileDesc*>(base + o_tiles);
    float* d_place = reinterpret_cast<float*>(base + o_place);
    float2* d_otf = reinterpret_cast<float2*>(base + o_otf);
    float2* d_spec = reinterpret_cast<float2*>(base + o_spec);
    const size_t smem_plane = 2 * (size_t)by.T * pitch * sizeof(float2);
    const size_t smem_z = 2 * (size_t)bz.T * kZPitch * sizeof(float2);

    // ---- kernel spectrum: placed kernel (cleared first), forward 3D FFT, scaled ----
    MVD_CHECK(cudaMemsetAsync(d_place, 0, (size_t)bx.T * by.T * bz.T * sizeof(float), s));
    const long long kn = (long long)kd[0] * kd[1] * kd[2];
    place_kernel_noalloc<<<(int)std::min<long long>((kn + 255) / 256, 4096), 256, 0, s>>>(
        kernel, kd[0], kd[1], kd[2], d_place, bx.T, by.T, bz.T);
    MVD_CHECK(cudaGetLastError());
    EpiBoxes no_boxes;  // no L2 prefetch: no tensor maps are built on this path
    std::memset(&no_boxes, 0, sizeof(no_boxes));
    set_smem(plane_fwd_kernel<GatherValue>, smem_plane);
    plane_fwd_kernel<GatherValue><<<(int)otf_fwd.size(), kThreads, smem_plane, s>>>(
        d_tiles, reinterpret_cast<const int2*>(base + o_ofwd), d_plans, d_otf,
        GatherValue::full(d_place, bx.T, by.T, bz.T, 0.f), no_boxes, 0);
    MVD_CHECK(cudaGetLastError());
    set_smem(zpass_kernel<1>, smem_z);
    zpass_kernel<1><<<(int)otf_z.size(), kZThreads, smem_z, s>>>(d_tiles, reinterpret_cast<const int2*>(base + o_oz),
                                                                 d_plans, d_otf, nullptr,
                                                                 (float)(1.0 / ((double)bx.T * by.T * bz.T)));
    MVD_CHECK(cudaGetLastError());

    // ---- the convolution: forward plane pass, z pass with the spectrum, inverse plane pass ----
    const int2* d_fwd = reinterpret_cast<const int2*>(base + o_fwd);
    if (ext_mode == 0) {
      set_smem(plane_fwd_kernel<GatherMirror>, smem_plane);
      plane_fwd_kernel<GatherMirror><<<(int)fwd.size(), kThreads, smem_plane, s>>>(
          d_tiles, d_fwd, d_plans, d_spec, GatherMirror{{in, nx, ny, nz}}, no_boxes, 0);
    } else {
      plane_fwd_kernel<GatherValue><<<(int)fwd.size(), kThreads, smem_plane, s>>>(
          d_tiles, d_fwd, d_plans, d_spec, GatherValue::full(in, nx, ny, nz, ext_value), no_boxes, 0);
    }
    MVD_CHECK(cudaGetLastError());
    set_smem(zpass_kernel<0>, smem_z);
    zpass_kernel<0><<<(int)zz.size(), kZThreads, smem_z, s>>>(d_tiles, reinterpret_cast<const int2*>(base + o_z),
                                                              d_plans, d_spec, d_otf, 1.f);
    MVD_CHECK(cudaGetLastError());
    if (!inv.empty()) {
      set_smem(plane_inv_kernel<EpiStore>, smem_plane);
      plane_inv_kernel<EpiStore><<<(int)inv.size(), kThreads, smem_plane, s>>>(
          d_tiles, reinterpret_cast<const int2*>(base + o_inv), d_plans, d_spec, EpiStore{out, nx, ny}, no_boxes);
      MVD_CHECK(cudaGetLastError());
    }
    count_launch(inv.empty() ? 5 : 6);
    return MVD_OK;
  } catch (const CudaError& e) {
    set_last_error(e.what());
    return MVD_ERR_CUDA;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return MVD_ERR_INTERNAL;
  }
}
