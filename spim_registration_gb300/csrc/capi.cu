// C ABI of libFourierConvolutionCUDA: the reference's JNA entry points and the
// whole-deconvolution handle.  Every entry point catches exceptions and turns them into a
// status code plus a per-thread message; nothing is retained across calls except in handles.
#include <algorithm>
#include <array>
#include <chrono>
#include <climits>
#include <cstdlib>
#include <cstdio>
#include <map>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/mvdecon.h"
#include "engine.h"

using namespace mvd;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int from_exception() {
  try {
    throw;
  } catch (const CudaError& e) {
    return fail(e.code == cudaErrorMemoryAllocation ? MVD_ERR_NOMEM : MVD_ERR_CUDA, e.what());
  } catch (const std::invalid_argument& e) {
    return fail(MVD_ERR_ARG, e.what());
  } catch (const std::bad_alloc&) {
    return fail(MVD_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(MVD_ERR_INTERNAL, e.what());
  } catch (...) {
    return fail(MVD_ERR_INTERNAL, "unknown error");
  }
}

#define MVD_API_BEGIN try {
#define MVD_API_END \
  }                 \
  catch (...) { return from_exception(); }

uint64_t fnv1a(const void* data, size_t bytes, uint64_t h = 1469598103934665603ULL) {
  const unsigned char* p = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < bytes; ++i) {
    h ^= p[i];
    h *= 1099511628211ULL;
  }
  return h;
}

// Per-device state of the drop-in convolution: stream, plans, cached kernel spectra.
struct DeviceCtx {
  std::mutex mu;
  int dev = -1;
  cudaStream_t stream = nullptr;
  PlanTable pt;
  std::map<std::vector<int>, std::unique_ptr<ConvPlan>> plans;
  struct Otf {
    DevBuf buf;
    uint64_t stamp;
    std::vector<float> kernel;  // the kernel's values: a hash match is confirmed against them
  };
  std::map<std::vector<uint64_t>, Otf> otfs;
  uint64_t clock = 0;
  DevBuf d_in, d_out, d_spec, d_kernel, scratch;

  ConvPlan& plan_for(int nx, int ny, int nz, int kx, int ky, int kz) {
    std::vector<int> key{nx, ny, nz, kx, ky, kz};
    auto it = plans.find(key);
    if (it != plans.end()) return *it->second;
    auto p = make_conv_plan(pt, nx, ny, nz, kx, ky, kz);
    ConvPlan& ref = *p;
    plans[key] = std::move(p);
    return ref;
  }

  // spectrum of a host kernel for a plan, cached by content (the Java side re-sends the same
  // kernel with every block: MVDeconFFTThreads.java:86-89).  The 64-bit hash only finds the
  // entry; a hit is used only when the kept kernel values equal the new ones.
  const float2* otf_for(const ConvPlan& plan, const float* host_kernel) {
    const size_t kn = (size_t)plan.kx * plan.ky * plan.kz;
    std::vector<uint64_t> key{fnv1a(host_kernel, kn * sizeof(float)), (uint64_t)plan.kx, (uint64_t)plan.ky,
                              (uint64_t)plan.kz, (uint64_t)plan.ax.T, (uint64_t)plan.ay.T, (uint64_t)plan.az.T};
    auto it = otfs.find(key);
    if (it != otfs.end()) {
      if (std::memcmp(it->second.kernel.data(), host_kernel, kn * sizeof(float)) == 0) {
        it->second.stamp = ++clock;
        return it->second.buf.as<float2>();
      }
      otfs.erase(it);  // another kernel with the same hash: its spectrum is rebuilt below
    }
    if (otfs.size() >= 16) {  // evict the least recently used spectrum
      auto victim = otfs.begin();
      for (auto i = otfs.begin(); i != otfs.end(); ++i)
        if (i->second.stamp < victim->second.stamp) victim = i;
      otfs.erase(victim);
    }
    d_kernel.ensure(kn * sizeof(float));
    MVD_CHECK(cudaMemcpyAsync(d_kernel.p, host_kernel, kn * sizeof(float), cudaMemcpyHostToDevice, stream));
    Otf o;
    o.buf.alloc(plan.otf_elems * sizeof(float2));
    build_otf(pt, plan, d_kernel.as<float>(), o.buf.as<float2>(), scratch, stream);
    o.stamp = ++clock;
    o.kernel.assign(host_kernel, host_kernel + kn);
    auto& slot = otfs[key];
    slot = std::move(o);
    return slot.buf.as<float2>();
  }
};

// MVD_TRACE=1 prints the duration of the phases of mvd_create and mvd_get_psi to stderr.
struct PhaseTrace {
  bool on;
  std::chrono::steady_clock::time_point t0;
  cudaStream_t s;
  explicit PhaseTrace(cudaStream_t st) : s(st) {
    const char* e = std::getenv("MVD_TRACE");
    on = e && *e == '1';
    t0 = std::chrono::steady_clock::now();
  }
  // the phase's wall time, and the part of it the host spent before waiting for the stream
  void mark(const char* what) {
    if (!on) return;
    auto th = std::chrono::steady_clock::now();
    cudaStreamSynchronize(s);
    auto t1 = std::chrono::steady_clock::now();
    std::fprintf(stderr, "[mvd] %-32s %8.2f ms (host %.2f ms)\n", what,
                 std::chrono::duration<double, std::milli>(t1 - t0).count(),
                 std::chrono::duration<double, std::milli>(th - t0).count());
    t0 = t1;
  }
};

// n side streams forked from `main`: each starts after the work enqueued so far on `main`,
// and join() makes `main` wait for all of them.  Streams and events are released when the
// object goes (CUDA frees them once their work is done); if join() was never reached (an
// error path), the side streams are waited for first, since buffers they use may be freed.
struct ForkedStreams {
  cudaStream_t main;
  std::vector<cudaStream_t> s;
  std::vector<cudaEvent_t> done;
  cudaEvent_t ready = nullptr;
  bool joined = false;
  ForkedStreams(cudaStream_t m, int n) : main(m) {
    MVD_CHECK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    MVD_CHECK(cudaEventRecord(ready, main));
    for (int i = 0; i < n; ++i) {
      cudaStream_t st;
      MVD_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
      s.push_back(st);
      cudaEvent_t e;
      MVD_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      done.push_back(e);
      MVD_CHECK(cudaStreamWaitEvent(st, ready, 0));
    }
  }
  void join() {
    for (size_t i = 0; i < s.size(); ++i) {
      MVD_CHECK(cudaEventRecord(done[i], s[i]));
      MVD_CHECK(cudaStreamWaitEvent(main, done[i], 0));
    }
    joined = true;
  }
  ~ForkedStreams() {
    for (size_t i = 0; i < s.size(); ++i) {
      if (!joined) cudaStreamSynchronize(s[i]);
      cudaEventDestroy(done[i]);
      cudaStreamDestroy(s[i]);
    }
    if (ready) cudaEventDestroy(ready);
  }
  ForkedStreams(const ForkedStreams&) = delete;
  ForkedStreams& operator=(const ForkedStreams&) = delete;
};

// whether copying from p returns before the copy is done (device memory, or host memory
// that is page-locked); a copy from pageable host memory holds the calling thread
bool async_copy_source(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged || a.type == cudaMemoryTypeHost;
}

std::mutex g_ctx_mu;
std::unordered_map<int, std::unique_ptr<DeviceCtx>> g_ctx;

DeviceCtx& ctx_for(int dev) {
  int count = 0;
  MVD_CHECK(cudaGetDeviceCount(&count));
  if (dev < 0 || dev >= count) throw std::invalid_argument("invalid CUDA device id");
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  auto& slot = g_ctx[dev];
  if (!slot) {
    auto c = std::make_unique<DeviceCtx>();
    c->dev = dev;
    MVD_CHECK(cudaSetDevice(dev));
    MVD_CHECK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    slot = std::move(c);
  }
  return *slot;
}

void check_dims(const int* d, const char* what) {
  if (!d) throw std::invalid_argument(std::string(what) + " is NULL");
  for (int i = 0; i < 3; ++i)
    if (d[i] < 1) throw std::invalid_argument(std::string(what) + " has a non-positive size");
}

}  // namespace

namespace mvd {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace mvd

// =========================================================================================
// Part 1: JNA interface
// =========================================================================================
extern "C" int getNumDevicesCUDA(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return n;
}

extern "C" int getCUDAcomputeCapabilityMajorVersion(int dev) {
  int v = -1;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess) return -1;
  return v;
}

extern "C" int getCUDAcomputeCapabilityMinorVersion(int dev) {
  int v = -1;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess) return -1;
  return v;
}

extern "C" void getNameDeviceCUDA(int dev, char* name) {
  if (!name) return;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    std::snprintf(name, 256, "unknown device %d", dev);
    return;
  }
  std::snprintf(name, 256, "%s", prop.name);
}

extern "C" long long getMemDeviceCUDA(int dev) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return -1;
  return (long long)prop.totalGlobalMem;
}

extern "C" long long getFreeMemDeviceCUDA(int dev) {
  int prev = 0;
  cudaGetDevice(&prev);
  if (cudaSetDevice(dev) != cudaSuccess) return -1;
  size_t fr = 0, tot = 0;
  cudaError_t e = cudaMemGetInfo(&fr, &tot);
  cudaSetDevice(prev);
  return e == cudaSuccess ? (long long)fr : -1;
}

extern "C" float* convolution3DfftCUDA(float*, int*, float*, int*, int) {
  fail(MVD_ERR_STATE, "convolution3DfftCUDA is not provided; use convolution3DfftCUDAInPlace");
  std::fprintf(stderr, "[FourierConvolutionCUDA] convolution3DfftCUDA is not provided; use convolution3DfftCUDAInPlace\n");
  return nullptr;
}

extern "C" const char* mvd_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* mvd_version(void) { return "mvdecon-gb300 0.1 (sm_103a)"; }

extern "C" int mvd_convolve3d_inplace(float* im, const int* imDim, const float* kernel, const int* kernelDim,
                                      int devCUDA) {
  MVD_API_BEGIN
  g_last_error.clear();
  check_dims(imDim, "imDim");
  check_dims(kernelDim, "kernelDim");
  if (!im || !kernel) return fail(MVD_ERR_ARG, "NULL image or kernel");
  const int nz = imDim[0], ny = imDim[1], nx = imDim[2];     // reversed: {z, y, x}
  const int kz = kernelDim[0], ky = kernelDim[1], kx = kernelDim[2];
  if (!(kx & 1) || !(ky & 1) || !(kz & 1)) return fail(MVD_ERR_ARG, "kernel sizes must be odd");
  DeviceCtx& c = ctx_for(devCUDA);
  std::lock_guard<std::mutex> lk(c.mu);
  MVD_CHECK(cudaSetDevice(devCUDA));
  ConvPlan& plan = c.plan_for(nx, ny, nz, kx, ky, kz);
  const size_t n = (size_t)nx * ny * nz;
  c.d_in.ensure(n * sizeof(float));
  c.d_out.ensure(n * sizeof(float));
  c.d_spec.ensure(plan.spec_elems * sizeof(float2));
  MVD_CHECK(cudaMemcpyAsync(c.d_in.p, im, n * sizeof(float), cudaMemcpyHostToDevice, c.stream));
  const float2* otf = c.otf_for(plan, kernel);
  convolve(c.pt, plan, c.d_in.as<float>(), Ext::Mirror, 0.f, otf, c.d_spec.as<float2>(), c.d_out.as<float>(),
           c.stream);
  // results only reach `im` once everything succeeded
  std::vector<float> tmp(n);
  MVD_CHECK(cudaMemcpyAsync(tmp.data(), c.d_out.p, n * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
  MVD_CHECK(cudaStreamSynchronize(c.stream));
  std::memcpy(im, tmp.data(), n * sizeof(float));
  return MVD_OK;
  MVD_API_END
}

extern "C" void convolution3DfftCUDAInPlace(float* im, int* imDim, float* kernel, int* kernelDim, int devCUDA) {
  const int st = mvd_convolve3d_inplace(im, imDim, kernel, kernelDim, devCUDA);
  if (st != MVD_OK)
    std::fprintf(stderr, "[FourierConvolutionCUDA] convolution3DfftCUDAInPlace failed (%d): %s\n", st,
                 g_last_error.c_str());
}

extern "C" int mvd_convolve3d_device(const float* in, float* out, const int* dims, const float* kernel,
                                     const int* kdims, int ext_mode, float ext_value, int devCUDA, void* stream) {
  MVD_API_BEGIN
  g_last_error.clear();
  check_dims(dims, "dims_xyz");
  check_dims(kdims, "kdims_xyz");
  if (!in || !out || !kernel) return fail(MVD_ERR_ARG, "NULL pointer");
  if (ext_mode != 0 && ext_mode != 1) return fail(MVD_ERR_ARG, "ext_mode must be 0 or 1");
  if (!(kdims[0] & 1) || !(kdims[1] & 1) || !(kdims[2] & 1)) return fail(MVD_ERR_ARG, "kernel sizes must be odd");
  DeviceCtx& c = ctx_for(devCUDA);
  std::lock_guard<std::mutex> lk(c.mu);
  MVD_CHECK(cudaSetDevice(devCUDA));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.stream;
  ConvPlan& plan = c.plan_for(dims[0], dims[1], dims[2], kdims[0], kdims[1], kdims[2]);
  c.d_spec.ensure(plan.spec_elems * sizeof(float2));
  DevBuf otf(plan.otf_elems * sizeof(float2));
  build_otf(c.pt, plan, kernel, otf.as<float2>(), c.scratch, s);
  convolve(c.pt, plan, in, ext_mode == 0 ? Ext::Mirror : Ext::Value, ext_value, otf.as<float2>(),
           c.d_spec.as<float2>(), out, s);
  // the spectrum buffers are reused by the next call: finish before returning
  MVD_CHECK(cudaStreamSynchronize(s));
  return MVD_OK;
  MVD_API_END
}

// =========================================================================================
// Part 2: deconvolution handle
// =========================================================================================
namespace {

constexpr int kHist = 64;

struct StatSlot {
  double sum;
  unsigned max_bits;
  unsigned ticket;  // CTAs of the view's update pass that are done (the last one archives)
};

// Copies the view's statistics into the history and clears its slot for the view's next
// update (the slots start cleared); after the last view the iteration counter advances.  The
// plain form runs it after its separate update kernel; the fused update pass does the same in
// its last CTA.
__global__ void archive_stats_kernel(StatSlot* slot, double* hist, int* iter, int view, int nviews) {
  const int it = *iter % kHist;
  hist[(it * nviews + view) * 2 + 0] = slot->sum;
  hist[(it * nviews + view) * 2 + 1] = (double)__uint_as_float(slot->max_bits);
  slot->sum = 0.0;
  slot->max_bits = 0u;
  if (view == nviews - 1) *iter += 1;
}

struct Block {
  int off[3], eoff[3], esz[3], local[3];
};

// BlockGeneratorFixedSizePrecise.divideIntoBlocks (BlockGeneratorFixedSizePrecise.java:46-122)
std::vector<Block> divide_into_blocks(const int img[3], const int k[3], const int b[3]) {
  int eff[3], nb[3];
  for (int d = 0; d < 3; ++d) {
    eff[d] = b[d] - k[d] + 1;
    if (eff[d] <= 0) throw std::invalid_argument("block size smaller than the kernel");
    nb[d] = img[d] / eff[d] + (img[d] % eff[d] ? 1 : 0);
  }
  std::vector<Block> out;
  for (int z = 0; z < nb[2]; ++z)
    for (int y = 0; y < nb[1]; ++y)
      for (int x = 0; x < nb[0]; ++x) {
        const int cur[3] = {x, y, z};
        Block bl;
        for (int d = 0; d < 3; ++d) {
          bl.eoff[d] = cur[d] * eff[d];
          bl.off[d] = bl.eoff[d] - k[d] / 2;
          bl.esz[d] = std::min(eff[d], img[d] - bl.eoff[d]);
          bl.local[d] = k[d] / 2;
        }
        out.push_back(bl);
      }
  return out;
}

}  // namespace

// Owns the handle's stream.  Declared first in mvd_decon, so it is destroyed last: every
// buffer of the handle is freed in this stream's order before the stream goes away.
struct StreamHolder {
  cudaStream_t s = nullptr;
  ~StreamHolder() {
    if (s) cudaStreamDestroy(s);
  }
};

struct mvd_decon {
  StreamHolder stream_holder;
  int dev = 0;
  cudaStream_t stream = nullptr;
  PlanTable pt;
  int dims[3] = {0, 0, 0};
  long long N = 0;
  int V = 0;
  int psftype = 0;
  float lambda = 0.f;
  int flags = 0;
  int ref_sum_threads = 0;  // AdjustInput.sumImg's thread count, 0 = plain sums
  std::vector<std::array<int, 3>> kd;
  DevBuf psi, q, tmp2, spec, scratch;
  std::vector<DevBuf> img, w, k1, k2, otf1, otf2;
  std::vector<std::unique_ptr<ConvPlan>> plans;
  // plain form
  int block[3] = {0, 0, 0};
  std::vector<std::vector<Block>> blocks;
  std::vector<std::array<int, 3>> block_size;
  DevBuf blk_in, blk_out;
  // statistics
  DevBuf stats, hist, d_iter, d_sc;
  int iteration = 0;
  double avg = 0.0;
  cudaGraphExec_t graph = nullptr;
  long long graph_kernels = 0;  // kernel launches one replay of the graph performs
  long long launches = 0;       // kernel launches issued by this handle

  ~mvd_decon() {
    if (graph) cudaGraphExecDestroy(graph);
  }

  // forward/backward of the image-formation model (allocated on first use)
  struct AdjView {
    std::unique_ptr<ConvPlan> ext;   // plan over the volume extended by k/2 (tiles shifted by -k/2)
    DevBuf otf_m;                    // spectrum of mirror(kernel1) on `ext`
    DevBuf fold_tab;                 // CSR tables of the mirror fold
    DevBuf lag_tile, lag_items_z, lag_items_inv;  // one full tile of the view's plan
    int n_lag_z = 0, n_lag_inv = 0;
  };
  std::vector<AdjView> adj;
  DevBuf r, c_ext, spec_ext, spec_b, acc, lag_real, g_psi, g_psf, d_nll;

  StatSlot* slot(int v) { return stats.as<StatSlot>() + v; }

  void enqueue_view(int v) {
    cudaStream_t s = stream;
    if (flags & MVD_FLAG_PLAIN) {
      enqueue_view_plain(v);
    } else {
      const ConvPlan& p = *plans[v];
      float2* sp = spec.as<float2>();
      launch_fwd_mirror(pt, p, psi.as<float>(), sp, s);
      launch_z(pt, p, sp, otf1[v].as<float2>(), s);
      launch_inv_quotient(pt, p, sp, img[v].as<float>(), q.as<float>(), s);
      launch_fwd_value(pt, p, q.as<float>(), 1.f, sp, s);
      launch_z(pt, p, sp, otf2[v].as<float2>(), s);
      launch_inv_update(pt, p, sp, psi.as<float>(), w[v].as<float>(), lambda, &slot(v)->sum, &slot(v)->max_bits,
                        archive(v), s);
    }
  }

  // the update pass's last CTA files view v's statistics (fused form)
  StatArchive archive(int v) {
    return StatArchive{hist.as<double>(), d_iter.as<int>(), &slot(v)->ticket, v, V, kHist};
  }

  // one block per launch sequence: copy block -> 3 FFT passes -> paste (MVDeconFFT.java:438-446,
  // 528-535, MVDeconFFTThreads.java:73-115), then separate quotient / update kernels
  void plain_conv(int v, const float* src, Ext ext, float value, const float2* otf, float* dst) {
    const ConvPlan& p = *plans[v];
    const auto& bs = block_size[v];
    for (const Block& b : blocks[v]) {
      dev_copy_block(src, dims[0], dims[1], dims[2], blk_in.as<float>(), bs[0], bs[1], bs[2], b.off[0], b.off[1],
                     b.off[2], ext, value, stream);
      convolve(pt, p, blk_in.as<float>(), Ext::Mirror, 0.f, otf, spec.as<float2>(), blk_out.as<float>(), stream);
      dev_paste_block(blk_out.as<float>(), bs[0], bs[1], bs[2], b.local[0], b.local[1], b.local[2], dst, dims[0],
                      dims[1], dims[2], b.eoff[0], b.eoff[1], b.eoff[2], b.esz[0], b.esz[1], b.esz[2], stream);
    }
  }

  void enqueue_view_plain(int v) {
    plain_conv(v, psi.as<float>(), Ext::Mirror, 0.f, otf1[v].as<float2>(), q.as<float>());
    dev_quotient(q.as<float>(), img[v].as<float>(), N, stream);
    plain_conv(v, q.as<float>(), Ext::Value, 1.f, otf2[v].as<float2>(), tmp2.as<float>());
    dev_update(psi.as<float>(), tmp2.as<float>(), w[v].as<float>(), lambda, N, &slot(v)->sum, &slot(v)->max_bits,
               stream);
    archive_stats_kernel<<<1, 1, 0, stream>>>(slot(v), hist.as<double>(), d_iter.as<int>(), v, V);
    MVD_CHECK(cudaGetLastError());
    count_launch();
  }

  void enqueue_iteration() {
    for (int v = 0; v < V; ++v) enqueue_view(v);
  }

  void run_iteration() {
    const bool use_graph = !(flags & (MVD_FLAG_PLAIN | MVD_FLAG_NO_GRAPH));
    if (use_graph) {
      if (!graph) {
        pt.device();  // no synchronous uploads may happen during capture
        cudaGraph_t g = nullptr;
        MVD_CHECK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        const long long before = launch_count();
        try {
          enqueue_iteration();
        } catch (...) {
          cudaStreamEndCapture(stream, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        MVD_CHECK(cudaStreamEndCapture(stream, &g));
        graph_kernels = launch_count() - before;
        cudaError_t e = cudaGraphInstantiate(&graph, g, 0);
        cudaGraphDestroy(g);
        MVD_CHECK(e);
      }
      MVD_CHECK(cudaGraphLaunch(graph, stream));
      launches += graph_kernels;
    } else {
      const long long before = launch_count();
      enqueue_iteration();
      launches += launch_count() - before;
    }
    ++iteration;
  }
};

namespace {

long long vox(const std::array<int, 3>& d) { return (long long)d[0] * d[1] * d[2]; }

DevBuf mirrored(mvd_decon* h, const float* k, const std::array<int, 3>& d) {
  DevBuf out(vox(d) * sizeof(float));
  dev_mirror(k, out.as<float>(), d[0], d[1], d[2], h->stream);
  return out;
}

// MVDeconFFT.init (MVDeconFFT.java:183-324) for every view, on the GPU and asynchronous: the
// PSF unit-sum normalisation in FP64 (AdjustInput.normImg, AdjustInput.java:50-56), the
// mirrored kernels and the compound kernels, whose small convolutions use zero extension
// (FFTConvolution over Views.extendZero, MVDeconFFT.java:222-248, 285-295).
void prepare_kernels(mvd_decon* h) {
  const int V = h->V;
  cudaStream_t s = h->stream;
  long long kmax = 0;
  for (int v = 0; v < V; ++v) kmax = std::max(kmax, vox(h->kd[v]));
  // AdjustInput.normImg: k /= sum(k), where the reference's sum counts portion 0 of
  // divideIntoPortions(n, 2 t) twice when run with t threads (AdjustInput.java:114-118)
  const int T = h->ref_sum_threads;
  auto norm_kernel = [T](float* k, long long n, double* sum, cudaStream_t st) {
    MVD_CHECK(cudaMemsetAsync(sum, 0, sizeof(double), st));
    dev_sum_f64(k, n, sum, st);
    if (T > 0) {
      const long long first = n / (2LL * T);  // portion 0 = [0, n / (2 t))
      if (first > 0) dev_sum_f64(k, first, sum, st);
    }
    dev_scale_div(k, n, sum, st);
  };
  // every view's compound kernel reads all normalised PSFs: normalise them first
  {
    DevBuf sum(sizeof(double));
    for (int v = 0; v < V; ++v) norm_kernel(h->k1[v].as<float>(), vox(h->kd[v]), sum.as<double>(), s);
  }
  // The plans of the PSF-pair convolutions (view v's PSF volume with view w's PSF) are built
  // here, with their tables uploaded in the handle stream's order, and each view gets scratch
  // sized for all of them, so that nothing is allocated while the views' chains run.
  const bool pairs = V > 1 && (h->psftype == MVD_EFFICIENT_BAYESIAN || h->psftype == MVD_OPTIMIZATION_I);
  std::map<std::vector<int>, std::unique_ptr<ConvPlan>> plans;
  size_t otf_max = 1, spec_max = 1, real_max = 1;
  auto plan_for = [&](const std::array<int, 3>& d, const std::array<int, 3>& kd) -> ConvPlan& {
    const std::vector<int> key{d[0], d[1], d[2], kd[0], kd[1], kd[2]};
    auto& plan = plans[key];
    if (!plan) {
      plan = make_conv_plan(h->pt, d[0], d[1], d[2], kd[0], kd[1], kd[2]);
      otf_max = std::max<size_t>(otf_max, plan->otf_elems);
      spec_max = std::max<size_t>(spec_max, plan->spec_elems);
      real_max = std::max<size_t>(real_max, (size_t)plan->ax.T * plan->ay.T * plan->az.T);
    }
    return *plan;
  };
  if (pairs)
    for (int v = 0; v < V; ++v)
      for (int wv = 0; wv < V; ++wv)
        if (wv != v) plan_for(h->kd[v], h->kd[wv]);
  h->pt.device();  // upload the FFT table with every length the plans added
  struct Scratch {
    DevBuf A, B, C, sum, otf, spec, real;
  };
  std::vector<Scratch> sc(V);
  for (int v = 0; v < V; ++v) {
    h->k2[v].alloc(vox(h->kd[v]) * sizeof(float));
    Scratch& x = sc[v];
    x.A.alloc(kmax * sizeof(float));
    x.B.alloc(kmax * sizeof(float));
    x.C.alloc(kmax * sizeof(float));
    x.sum.alloc(sizeof(double));
    if (pairs) {
      x.otf.alloc(otf_max * sizeof(float2));
      x.spec.alloc(spec_max * sizeof(float2));
      x.real.alloc(real_max * sizeof(float));
    }
  }
  // Each view's chain of small launches runs on its own stream: the chains are independent
  // and their kernels are far too small to fill the GPU one at a time.
  ForkedStreams fork(s, V);
  for (int v = 0; v < V; ++v) {
    cudaStream_t st = fork.s[v];
    Scratch& x = sc[v];
    const auto& dv = h->kd[v];
    const long long nv = vox(dv);
    float* k2 = h->k2[v].as<float>();
    const float* k1 = h->k1[v].as<float>();
    auto norm = [&](float* k) { norm_kernel(k, nv, x.sum.as<double>(), st); };
    // out = ext0(in) (*) kern over in's dims
    auto conv0 = [&](const float* in, const float* kern, const std::array<int, 3>& kd, float* out) {
      ConvPlan& plan = plan_for(dv, kd);
      build_otf(h->pt, plan, kern, x.otf.as<float2>(), x.real, st);
      convolve(h->pt, plan, in, Ext::Value, 0.f, x.otf.as<float2>(), x.spec.as<float2>(), out, st);
    };
    if (V == 1 || h->psftype == MVD_INDEPENDENT) {
      dev_mirror(k1, k2, dv[0], dv[1], dv[2], st);
    } else if (h->psftype == MVD_EFFICIENT_BAYESIAN) {
      // P_v^compound = P_v* prod_{w != v} crop(crop(P_v* (*) P_w) (*) P_w*)
      dev_mirror(k1, k2, dv[0], dv[1], dv[2], st);
      for (int wv = 0; wv < V; ++wv) {
        if (wv == v) continue;
        const auto& dw = h->kd[wv];
        dev_mirror(k1, x.A.as<float>(), dv[0], dv[1], dv[2], st);
        conv0(x.A.as<float>(), h->k1[wv].as<float>(), dw, x.B.as<float>());
        dev_mirror(h->k1[wv].as<float>(), x.C.as<float>(), dw[0], dw[1], dw[2], st);
        conv0(x.B.as<float>(), x.C.as<float>(), dw, x.A.as<float>());
        dev_mul(k2, x.A.as<float>(), nv, st);
      }
      norm(k2);
    } else if (h->psftype == MVD_OPTIMIZATION_I) {
      // mirror(norm(P_v prod_{w != v} crop(P_v (*) P_w*)))
      MVD_CHECK(cudaMemcpyAsync(x.A.p, k1, nv * sizeof(float), cudaMemcpyDeviceToDevice, st));
      for (int wv = 0; wv < V; ++wv) {
        if (wv == v) continue;
        const auto& dw = h->kd[wv];
        dev_mirror(h->k1[wv].as<float>(), x.C.as<float>(), dw[0], dw[1], dw[2], st);
        conv0(k1, x.C.as<float>(), dw, x.B.as<float>());
        dev_mul(x.A.as<float>(), x.B.as<float>(), nv, st);
      }
      norm(x.A.as<float>());
      dev_mirror(x.A.as<float>(), k2, dv[0], dv[1], dv[2], st);
    } else {
      // OPTIMIZATION_II: mirror(norm(P_v ^ V))
      MVD_CHECK(cudaMemcpyAsync(x.A.p, k1, nv * sizeof(float), cudaMemcpyDeviceToDevice, st));
      dev_pow(x.A.as<float>(), V, nv, st);
      norm(x.A.as<float>());
      dev_mirror(x.A.as<float>(), k2, dv[0], dv[1], dv[2], st);
    }
  }
  fork.join();
  // the scratch buffers and plans go out of scope after the join: freed in the handle
  // stream's order, behind the views' chains
}

// A view's convolutions only need to cover the bounding box of its data or weight (img > 0
// or w > 0): outside it the quotient is 1 (MVDeconvolution.java:519-522) and the update leaves
// psi unchanged (weight 0, :723).  The boxes come from dev_data_box in mvd_create.
// Tile plan of a view over its data box; with `autotune` the plane budgets below, each with
// 384- and 256-thread plane CTAs, are all tried and the fastest plan (one timed view stage
// each) is kept.  More warps hide more latency; fewer threads leave fewer idle at the stages'
// last butterfly round, which wins for some plane shapes.
// The autotuner's choices, kept for the process: an acquisition deconvolves job after job with
// the same geometry, so only the first job pays for the timing runs.  Keyed by device, data-box
// size, kernel size and the tensor-core flag.
struct TunedChoice {
  int cap, threads;
  bool generic, ascending, staged;
};
std::mutex g_tuned_mu;
std::map<std::array<int, 8>, TunedChoice> g_tuned;

std::unique_ptr<ConvPlan> plan_view(mvd_decon* h, int v, const int lo[3], const int hi[3], bool autotune,
                                    bool tensor_dft) {
  const auto& k = h->kd[v];
  const int n[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  const bool full = lo[0] == 0 && lo[1] == 0 && lo[2] == 0 && hi[0] == h->dims[0] && hi[1] == h->dims[1] &&
                    hi[2] == h->dims[2];
  auto make = [&](int cap, bool ascending) {
    PlanOptions o;
    o.cap = cap;
    o.ascending = ascending;
    auto p = make_conv_plan(h->pt, n[0], n[1], n[2], k[0], k[1], k[2], o);
    if (!full) place_plan(*p, lo[0], lo[1], lo[2], h->dims);
    p->tensor_dft = tensor_dft;
    return p;
  };
  if (!autotune) return make(0, false);
  const std::array<int, 8> key{h->dev, n[0], n[1], n[2], k[0], k[1], k[2], tensor_dft ? 1 : 0};
  {
    std::lock_guard<std::mutex> lock(g_tuned_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      auto p = make(it->second.cap, it->second.ascending);
      p->threads_plane = it->second.threads;
      p->generic = it->second.generic || it->second.ascending;
      p->staged = it->second.staged;
      return p;
    }
  }
  // one view stage of a candidate (two convolutions' passes), best of 3 after a warm-up
  cudaEvent_t e0, e1;
  MVD_CHECK(cudaEventCreate(&e0));
  MVD_CHECK(cudaEventCreate(&e1));
  auto time_stage = [&](ConvPlan& p, DevBuf& otf, DevBuf& spec) {
    float ms = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
      MVD_CHECK(cudaEventRecord(e0, h->stream));
      launch_fwd_mirror(h->pt, p, h->psi.as<float>(), spec.as<float2>(), h->stream);
      launch_z(h->pt, p, spec.as<float2>(), otf.as<float2>(), h->stream);
      launch_inv_quotient(h->pt, p, spec.as<float2>(), h->img[v].as<float>(), h->q.as<float>(), h->stream);
      launch_fwd_value(h->pt, p, h->q.as<float>(), 1.f, spec.as<float2>(), h->stream);
      launch_z(h->pt, p, spec.as<float2>(), otf.as<float2>(), h->stream);
      launch_inv_quotient(h->pt, p, spec.as<float2>(), h->img[v].as<float>(), h->q.as<float>(), h->stream);
      MVD_CHECK(cudaEventRecord(e1, h->stream));
      MVD_CHECK(cudaEventSynchronize(e1));
      float t = 0.f;
      MVD_CHECK(cudaEventElapsedTime(&t, e0, e1));
      if (rep > 0) ms = std::min(ms, t);
    }
    return ms;
  };
  // Candidates: the tile shapes of four plane budgets; for each, the default kernels (the
  // compiled ones where the shape has them), the generic kernels at 384 threads (where compiled
  // ones exist) and at 256 threads, and the generic kernels with every length's radices in
  // ascending order (a second radix plan of the same lengths).
  std::unique_ptr<ConvPlan> best;
  TunedChoice best_choice{0, kThreads, false, false, false};
  float best_ms = 1e30f;
  std::vector<std::array<int, 3>> seen;
  for (int cap : {4608, 7168, 10240, 14336}) {
    auto p = make(cap, false);
    const std::array<int, 3> shape{p->ax.T, p->ay.T, p->az.T};
    if (std::find(seen.begin(), seen.end(), shape) != seen.end()) continue;
    seen.push_back(shape);
    DevBuf otf(p->otf_elems * sizeof(float2)), spec(p->spec_elems * sizeof(float2));
    MVD_CHECK(cudaMemsetAsync(otf.p, 0, otf.bytes, h->stream));
    struct Variant {
      int threads;
      bool generic, staged;
    };
    // the tensor-core z pass runs with the compiled kernels only: with it asked for, they (and
    // their in-place variant) are the variants timed (the generic and ascending-radix
    // candidates would drop it)
    std::vector<Variant> variants{{kThreads, false, false}};
    p->staged = true;
    if (has_staged_kernels(*p)) variants.push_back({kThreads, false, true});
    p->staged = false;
    if (!tensor_dft) {
      variants.push_back({256, true, false});
      if (has_compiled_kernels(*p)) variants.push_back({kThreads, true, false});
    }
    float ms = 1e30f;
    Variant bv = variants[0];
    for (const Variant& var : variants) {
      p->threads_plane = var.threads;
      p->generic = var.generic;
      p->staged = var.staged;
      const float t = time_stage(*p, otf, spec);
      if (t < ms) {
        ms = t;
        bv = var;
      }
    }
    p->threads_plane = bv.threads;
    p->generic = bv.generic;
    p->staged = bv.staged;
    if (!tensor_dft) {
      auto asc = make(cap, true);
      const float t_asc = time_stage(*asc, otf, spec);
      if (t_asc < ms) {
        ms = t_asc;
        p = std::move(asc);
      }
    }
    if (ms < best_ms) {
      best_ms = ms;
      best_choice = TunedChoice{cap, p->threads_plane, p->generic, p->ascending, p->staged};
      best = std::move(p);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  std::lock_guard<std::mutex> lock(g_tuned_mu);
  g_tuned[key] = best_choice;
  return best;
}

std::unique_ptr<ConvPlan> block_plan(PlanTable& pt, const std::array<int, 3>& b, const std::array<int, 3>& k) {
  // the block convolved as a volume (mirror-single at its own border); its interior is what
  // the paste consumes
  return make_conv_plan(pt, b[0], b[1], b[2], k[0], k[1], k[2]);
}

// view v's kernel spectra (PSF and compound kernel) on its plan's padded tile grid
void build_view_otfs(mvd_decon* h, int v) {
  const ConvPlan& p = *h->plans[v];
  h->otf1[v].alloc(p.otf_elems * sizeof(float2));
  h->otf2[v].alloc(p.otf_elems * sizeof(float2));
  build_otf(h->pt, p, h->k1[v].as<float>(), h->otf1[v].as<float2>(), h->scratch, h->stream);
  build_otf(h->pt, p, h->k2[v].as<float>(), h->otf2[v].as<float2>(), h->scratch, h->stream);
}

}  // namespace

extern "C" int mvd_create(mvd_decon** out, int devCUDA, const int* dims, int num_views, const float* const* views,
                          const float* const* weights, const float* const* psfs, const int* psf_dims, int psftype,
                          double lambda, int flags, const int* block_xyz) {
  MVD_API_BEGIN
  g_last_error.clear();
  if (!out) return fail(MVD_ERR_ARG, "out is NULL");
  *out = nullptr;
  check_dims(dims, "dims_xyz");
  if (num_views < 1 || num_views > 16) return fail(MVD_ERR_ARG, "num_views must be in [1, 16]");
  if (!views || !weights || !psfs || !psf_dims) return fail(MVD_ERR_ARG, "NULL input array");
  if (psftype < 0 || psftype > 3) return fail(MVD_ERR_ARG, "unknown psftype");
  for (int v = 0; v < num_views; ++v) {
    if (!views[v] || !weights[v] || !psfs[v]) return fail(MVD_ERR_ARG, "NULL view, weight or psf");
    check_dims(psf_dims + 3 * v, "psf_dims");
    for (int d = 0; d < 3; ++d)
      if (!(psf_dims[3 * v + d] & 1)) return fail(MVD_ERR_ARG, "psf sizes must be odd");
  }
  if (block_xyz) check_dims(block_xyz, "block_xyz");
  int count = 0;
  MVD_CHECK(cudaGetDeviceCount(&count));
  if (devCUDA < 0 || devCUDA >= count) return fail(MVD_ERR_ARG, "invalid CUDA device id");
  MVD_CHECK(cudaSetDevice(devCUDA));
  auto h = std::make_unique<mvd_decon>();
  h->dev = devCUDA;
  MVD_CHECK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  h->stream_holder.s = h->stream;
  // the handle's buffers, plans and temporaries come from the device pool in stream order
  keep_pool_memory(devCUDA);
  AllocScope scope(h->stream);
  for (int d = 0; d < 3; ++d) h->dims[d] = dims[d];
  h->N = (long long)dims[0] * dims[1] * dims[2];
  h->V = num_views;
  h->psftype = psftype;
  h->lambda = (float)lambda;
  h->flags = flags;
  h->ref_sum_threads = (int)(((unsigned)flags >> 16) & 0x7fffu);
  const size_t nb = h->N * sizeof(float);
  h->img.resize(num_views);
  h->w.resize(num_views);
  h->k1.resize(num_views);
  h->k2.resize(num_views);
  h->otf1.resize(num_views);
  h->otf2.resize(num_views);
  PhaseTrace trace(h->stream);
  for (int v = 0; v < num_views; ++v) {
    h->kd.push_back({psf_dims[3 * v], psf_dims[3 * v + 1], psf_dims[3 * v + 2]});
    h->img[v].alloc(nb);
    h->w[v].alloc(nb);
    const size_t kb = vox(h->kd[v]) * sizeof(float);
    h->k1[v].alloc(kb);
    // cudaMemcpyDefault: the inputs may be host memory or device memory (for example views
    // resampled on the GPU by mvd_transform_view); unified addressing tells them apart
    MVD_CHECK(cudaMemcpyAsync(h->k1[v].p, psfs[v], kb, cudaMemcpyDefault, h->stream));
  }
  // The compound kernels need only the PSFs, so they run while the views and weights are
  // copied on a side stream.  The buffers were allocated in the handle stream's order, so the
  // copy stream starts after that point, and the handle stream waits for the copies before its
  // first use of the data.  Copies from device or page-locked memory return at once and are
  // enqueued first; a copy from pageable memory holds the host until it is done, so the
  // kernels are enqueued before those.
  bool async_src = true;
  for (int v = 0; v < num_views; ++v)
    async_src = async_src && async_copy_source(views[v]) && async_copy_source(weights[v]);
  ForkedStreams up(h->stream, 1);
  auto copy_inputs = [&] {
    for (int v = 0; v < num_views; ++v) {
      MVD_CHECK(cudaMemcpyAsync(h->img[v].p, views[v], nb, cudaMemcpyDefault, up.s[0]));
      MVD_CHECK(cudaMemcpyAsync(h->w[v].p, weights[v], nb, cudaMemcpyDefault, up.s[0]));
    }
  };
  if (async_src) copy_inputs();
  prepare_kernels(h.get());
  trace.mark("kernel preparation");
  if (!async_src) copy_inputs();
  up.join();
  trace.mark("input upload (rest of it)");
  h->psi.alloc(nb);
  h->q.alloc(nb);
  MVD_CHECK(cudaMemsetAsync(h->psi.p, 0, nb, h->stream));
  MVD_CHECK(cudaMemsetAsync(h->q.p, 0, nb, h->stream));
  long long spec_max = 0;
  if (flags & MVD_FLAG_PLAIN) {
    h->tmp2.alloc(nb);
    size_t blk_max = 0;
    for (int v = 0; v < num_views; ++v) {
      std::array<int, 3> bs;
      for (int d = 0; d < 3; ++d) bs[d] = block_xyz ? block_xyz[d] : dims[d] + h->kd[v][d] - 1;
      h->block_size.push_back(bs);
      h->blocks.push_back(divide_into_blocks(h->dims, h->kd[v].data(), bs.data()));
      h->plans.push_back(block_plan(h->pt, bs, h->kd[v]));
      blk_max = std::max<size_t>(blk_max, (size_t)vox(bs));
    }
    h->blk_in.alloc(blk_max * sizeof(float));
    h->blk_out.alloc(blk_max * sizeof(float));
  } else {
    // data boxes of all views (GPU reduction), then one plan per view
    std::vector<int> boxes(6 * num_views);
    for (int v = 0; v < num_views; ++v) {
      const int init[6] = {INT_MAX, INT_MAX, INT_MAX, -1, -1, -1};
      std::copy(init, init + 6, boxes.begin() + 6 * v);
    }
    DevBuf d_boxes(boxes.size() * sizeof(int));
    MVD_CHECK(cudaMemcpyAsync(d_boxes.p, boxes.data(), boxes.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    for (int v = 0; v < num_views; ++v)
      dev_data_box(h->img[v].as<float>(), h->w[v].as<float>(), dims[0], dims[1], dims[2], d_boxes.as<int>() + 6 * v,
                   h->stream);
    MVD_CHECK(cudaMemcpyAsync(boxes.data(), d_boxes.p, boxes.size() * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MVD_CHECK(cudaStreamSynchronize(h->stream));
    for (int v = 0; v < num_views; ++v) {
      int lo[3], hi[3];
      const int* b = boxes.data() + 6 * v;
      const bool empty = b[3] < 0;  // no data and no weight: the whole volume (a no-op view)
      for (int d = 0; d < 3; ++d) {
        lo[d] = empty ? 0 : b[d];
        hi[d] = empty ? dims[d] : b[3 + d] + 1;
      }
      if (flags & MVD_FLAG_TENSOR_DFT) tensor_dft_prepare();
      h->plans.push_back(plan_view(h.get(), v, lo, hi, (flags & MVD_FLAG_AUTOTUNE) != 0,
                                   (flags & MVD_FLAG_TENSOR_DFT) != 0));
      // the view's kernel spectra run on the GPU while the host plans the next view
      build_view_otfs(h.get(), v);
    }
  }
  if (flags & MVD_FLAG_PLAIN)
    for (int v = 0; v < num_views; ++v) build_view_otfs(h.get(), v);
  for (int v = 0; v < num_views; ++v) spec_max = std::max(spec_max, h->plans[v]->spec_elems);
  h->spec.alloc(spec_max * sizeof(float2));
  h->scratch.alloc(0);
  trace.mark("tile plans and kernel spectra");
  // first iteration: psi := average intensity of the overlapping area
  h->d_sc.alloc(2 * sizeof(double));
  MVD_CHECK(cudaMemsetAsync(h->d_sc.p, 0, 2 * sizeof(double), h->stream));
  std::vector<const float*> vp;
  for (int v = 0; v < num_views; ++v) vp.push_back(h->img[v].as<float>());
  dev_first_iteration(vp.data(), num_views, h->N, h->d_sc.as<double>(), h->stream);
  dev_fill_from_avg(h->psi.as<float>(), h->d_sc.as<double>(), h->N, h->stream);
  double sc[2];
  MVD_CHECK(cudaMemcpyAsync(sc, h->d_sc.p, sizeof(sc), cudaMemcpyDeviceToHost, h->stream));
  h->stats.alloc(num_views * sizeof(StatSlot));
  h->hist.alloc((size_t)kHist * num_views * 2 * sizeof(double));
  h->d_iter.alloc(sizeof(int));
  MVD_CHECK(cudaMemsetAsync(h->stats.p, 0, num_views * sizeof(StatSlot), h->stream));
  MVD_CHECK(cudaMemsetAsync(h->hist.p, 0, (size_t)kHist * num_views * 2 * sizeof(double), h->stream));
  MVD_CHECK(cudaMemsetAsync(h->d_iter.p, 0, sizeof(int), h->stream));
  MVD_CHECK(cudaStreamSynchronize(h->stream));
  h->avg = sc[0] / sc[1];
  if (h->avg != h->avg) h->avg = 0.5;
  trace.mark("first iteration, buffers");
  *out = h.release();
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_destroy(mvd_decon* h) {
  MVD_API_BEGIN
  if (!h) return MVD_OK;
  cudaSetDevice(h->dev);
  if (h->stream) cudaStreamSynchronize(h->stream);
  delete h;
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_run_view(mvd_decon* h, int view) {
  MVD_API_BEGIN
  if (!h) return fail(MVD_ERR_ARG, "NULL handle");
  if (view < 0 || view >= h->V) return fail(MVD_ERR_ARG, "view out of range");
  MVD_CHECK(cudaSetDevice(h->dev));
  h->enqueue_view(view);  // the last view's archive advances the device-side counter
  if (view == h->V - 1) ++h->iteration;
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_run_iteration(mvd_decon* h) {
  MVD_API_BEGIN
  if (!h) return fail(MVD_ERR_ARG, "NULL handle");
  MVD_CHECK(cudaSetDevice(h->dev));
  h->run_iteration();
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_run(mvd_decon* h, int iterations) {
  MVD_API_BEGIN
  if (!h) return fail(MVD_ERR_ARG, "NULL handle");
  if (iterations < 0) return fail(MVD_ERR_ARG, "negative iteration count");
  MVD_CHECK(cudaSetDevice(h->dev));
  for (int i = 0; i < iterations; ++i) h->run_iteration();
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_synchronize(mvd_decon* h) {
  MVD_API_BEGIN
  if (!h) return fail(MVD_ERR_ARG, "NULL handle");
  MVD_CHECK(cudaSetDevice(h->dev));
  MVD_CHECK(cudaStreamSynchronize(h->stream));
  // a tensor-core z pass whose bounded wait gave up left its CTA's pencils uncomputed
  if (h->flags & MVD_FLAG_TENSOR_DFT)
    if (const int n = tensor_dft_failures())
      return fail(MVD_ERR_CUDA, std::to_string(n) + " tensor-core DFT stages gave up waiting for their products");
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_get_psi(mvd_decon* h, float* psi, int masked) {
  MVD_API_BEGIN
  if (!h || !psi) return fail(MVD_ERR_ARG, "NULL argument");
  MVD_CHECK(cudaSetDevice(h->dev));
  const size_t nb = h->N * sizeof(float);
  if (masked) {
    PhaseTrace trace(h->stream);
    trace.mark("get_psi: pending work");
    // the quotient buffer is idle between view stages (every stage rewrites it before use):
    // the masked copy is staged there instead of in a fresh allocation
    MVD_CHECK(cudaMemcpyAsync(h->q.p, h->psi.p, nb, cudaMemcpyDeviceToDevice, h->stream));
    std::vector<const float*> vp;
    for (int v = 0; v < h->V; ++v) vp.push_back(h->img[v].as<float>());
    dev_mask(h->q.as<float>(), vp.data(), h->V, h->N, h->stream);
    trace.mark("get_psi: mask");
    MVD_CHECK(cudaMemcpyAsync(psi, h->q.p, nb, cudaMemcpyDeviceToHost, h->stream));
    MVD_CHECK(cudaStreamSynchronize(h->stream));
    trace.mark("get_psi: download");
  } else {
    MVD_CHECK(cudaMemcpyAsync(psi, h->psi.p, nb, cudaMemcpyDeviceToHost, h->stream));
    MVD_CHECK(cudaStreamSynchronize(h->stream));
  }
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_set_psi(mvd_decon* h, const float* psi) {
  MVD_API_BEGIN
  if (!h || !psi) return fail(MVD_ERR_ARG, "NULL argument");
  MVD_CHECK(cudaSetDevice(h->dev));
  MVD_CHECK(cudaMemcpyAsync(h->psi.p, psi, h->N * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  MVD_CHECK(cudaStreamSynchronize(h->stream));
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_get_initial_average(mvd_decon* h, double* avg) {
  if (!h || !avg) return fail(MVD_ERR_ARG, "NULL argument");
  *avg = h->avg;
  return MVD_OK;
}

extern "C" int mvd_get_kernel(mvd_decon* h, int view, int which, float* out) {
  MVD_API_BEGIN
  if (!h || !out) return fail(MVD_ERR_ARG, "NULL argument");
  if (view < 0 || view >= h->V || (which != 1 && which != 2)) return fail(MVD_ERR_ARG, "bad view or kernel");
  MVD_CHECK(cudaSetDevice(h->dev));
  const DevBuf& k = which == 1 ? h->k1[view] : h->k2[view];
  MVD_CHECK(cudaMemcpyAsync(out, k.p, vox(h->kd[view]) * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  MVD_CHECK(cudaStreamSynchronize(h->stream));
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_get_stats(mvd_decon* h, int iteration, int view, double* sum_change, double* max_change) {
  MVD_API_BEGIN
  if (!h || !sum_change || !max_change) return fail(MVD_ERR_ARG, "NULL argument");
  if (view < 0 || view >= h->V) return fail(MVD_ERR_ARG, "view out of range");
  if (iteration < 0 || iteration >= h->iteration + 1 || iteration < h->iteration + 1 - kHist)
    return fail(MVD_ERR_ARG, "iteration not in the kept history");
  MVD_CHECK(cudaSetDevice(h->dev));
  double v2[2];
  const int it = iteration % kHist;
  MVD_CHECK(cudaMemcpyAsync(v2, h->hist.as<double>() + (it * h->V + view) * 2, sizeof(v2), cudaMemcpyDeviceToHost,
                            h->stream));
  MVD_CHECK(cudaStreamSynchronize(h->stream));
  *sum_change = v2[0];
  *max_change = v2[1];
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_get_iteration(mvd_decon* h, int* iteration) {
  if (!h || !iteration) return fail(MVD_ERR_ARG, "NULL argument");
  *iteration = h->iteration;
  return MVD_OK;
}

extern "C" int mvd_get_plan(mvd_decon* h, int view, int* tiles, int* tile, int* eff, long long* padded) {
  if (!h) return fail(MVD_ERR_ARG, "NULL handle");
  if (view < 0 || view >= h->V) return fail(MVD_ERR_ARG, "view out of range");
  const ConvPlan& p = *h->plans[view];
  const AxisTiles* a[3] = {&p.ax, &p.ay, &p.az};
  for (int d = 0; d < 3; ++d) {
    if (tiles) tiles[d] = a[d]->n;
    if (tile) tile[d] = a[d]->T;
    if (eff) eff[d] = a[d]->E;
  }
  if (padded) {
    long long pv = p.padded_voxels();
    if (h->flags & MVD_FLAG_PLAIN) pv *= (long long)h->blocks[view].size();
    *padded = pv;
  }
  return MVD_OK;
}

extern "C" int mvd_get_plan_variant(mvd_decon* h, int view, int* threads, int* variant) {
  if (!h) return fail(MVD_ERR_ARG, "NULL handle");
  if (view < 0 || view >= h->V) return fail(MVD_ERR_ARG, "view out of range");
  const ConvPlan& p = *h->plans[view];
  const bool compiled = !p.generic && has_compiled_kernels(p) && p.threads_plane == kThreads;
  const bool staged = compiled && p.staged && has_staged_kernels(p);
  if (threads) *threads = staged ? 512 : compiled && compiled_plane_threads(p) ? compiled_plane_threads(p) : p.threads_plane;
  if (variant)
    *variant = (compiled ? 1 : 0) | (p.ascending ? 2 : 0) |
               (p.tensor_dft && !p.generic && tensor_dft_supported(p.az.T) ? 4 : 0) | (staged ? 8 : 0);
  return MVD_OK;
}

extern "C" int mvd_get_stream(mvd_decon* h, void** stream) {
  if (!h || !stream) return fail(MVD_ERR_ARG, "NULL argument");
  *stream = (void*)h->stream;
  return MVD_OK;
}

extern "C" int mvd_get_launch_count(mvd_decon* h, long long* launches) {
  if (!h || !launches) return fail(MVD_ERR_ARG, "NULL argument");
  *launches = h->launches;
  return MVD_OK;
}

extern "C" int mvd_profile_iteration(mvd_decon* h, double* ms, int* launches) {
  MVD_API_BEGIN
  if (!h || !ms || !launches) return fail(MVD_ERR_ARG, "NULL argument");
  if (h->flags & MVD_FLAG_PLAIN) return fail(MVD_ERR_STATE, "pass profiling needs the fused form");
  MVD_CHECK(cudaSetDevice(h->dev));
  cudaStream_t s = h->stream;
  const int kinds = 5;
  std::vector<cudaEvent_t> ev;
  std::vector<int> kind;
  auto mark = [&](int k) {
    cudaEvent_t e;
    MVD_CHECK(cudaEventCreate(&e));
    MVD_CHECK(cudaEventRecord(e, s));
    ev.push_back(e);
    kind.push_back(k);
  };
  for (int k = 0; k < kinds; ++k) {
    ms[k] = 0.0;
    launches[k] = 0;
  }
  mark(-1);
  for (int v = 0; v < h->V; ++v) {
    const ConvPlan& p = *h->plans[v];
    float2* sp = h->spec.as<float2>();
    launch_fwd_mirror(h->pt, p, h->psi.as<float>(), sp, s);
    mark(0);
    launch_z(h->pt, p, sp, h->otf1[v].as<float2>(), s);
    mark(1);
    launch_inv_quotient(h->pt, p, sp, h->img[v].as<float>(), h->q.as<float>(), s);
    mark(2);
    launch_fwd_value(h->pt, p, h->q.as<float>(), 1.f, sp, s);
    mark(0);
    launch_z(h->pt, p, sp, h->otf2[v].as<float2>(), s);
    mark(1);
    launch_inv_update(h->pt, p, sp, h->psi.as<float>(), h->w[v].as<float>(), h->lambda, &h->slot(v)->sum,
                      &h->slot(v)->max_bits, h->archive(v), s);
    mark(3);
  }
  MVD_CHECK(cudaStreamSynchronize(s));
  for (size_t i = 1; i < ev.size(); ++i) {
    float t = 0.f;
    MVD_CHECK(cudaEventElapsedTime(&t, ev[i - 1], ev[i]));
    ms[kind[i]] += t;
    launches[kind[i]] += 1;
  }
  for (auto e : ev) cudaEventDestroy(e);
  ++h->iteration;
  h->launches += 6 * h->V;
  return MVD_OK;
  MVD_API_END
}

// =========================================================================================
// forward / backward pair of the multiview Poisson image-formation model
// (no counterpart in the reference: gradients for PSF refinement from bead data)
// =========================================================================================
namespace {

void adjoint_setup(mvd_decon* h) {
  if (!h->adj.empty()) return;
  AllocScope scope(h->stream);
  h->adj.resize(h->V);
  long long ext_max = 0, spec_ext_max = 0, tile_max = 0, otf_max = 0;
  for (int v = 0; v < h->V; ++v) {
    mvd_decon::AdjView& a = h->adj[v];
    const auto& k = h->kd[v];
    const int hx = k[0] / 2, hy = k[1] / 2, hz = k[2] / 2;
    const int nxe = h->dims[0] + 2 * hx, nye = h->dims[1] + 2 * hy, nze = h->dims[2] + 2 * hz;
    a.ext = make_conv_plan(h->pt, nxe, nye, nze, k[0], k[1], k[2]);
    for (auto& t : a.ext->tiles) {  // tile coordinates in the original volume's frame
      t.ox -= hx;
      t.oy -= hy;
      t.oz -= hz;
    }
    a.ext->upload();
    ext_max = std::max(ext_max, (long long)nxe * nye * nze);
    spec_ext_max = std::max(spec_ext_max, a.ext->spec_elems);
    DevBuf mk = mirrored(h, h->k1[v].as<float>(), k);
    a.otf_m.alloc(a.ext->otf_elems * sizeof(float2));
    build_otf(h->pt, *a.ext, mk.as<float>(), a.otf_m.as<float2>(), h->scratch, h->stream);
    std::vector<int> tab, st, ix;
    const int n3[3] = {h->dims[0], h->dims[1], h->dims[2]}, h3[3] = {hx, hy, hz};
    for (int d = 0; d < 3; ++d) {
      mirror_fold_table(n3[d], h3[d], st, ix);
      tab.insert(tab.end(), st.begin(), st.end());
      tab.insert(tab.end(), ix.begin(), ix.end());
    }
    a.fold_tab.alloc(tab.size() * sizeof(int));
    upload_table(a.fold_tab.p, tab.data(), tab.size() * sizeof(int));
    // one full tile of the view's plan, for the inverse transform of the accumulated spectrum
    const ConvPlan& p = *h->plans[v];
    TileDesc t = p.tiles[0];
    t.ox = t.oy = t.oz = 0;
    t.hx = t.hy = t.hz = 0;
    t.ex = p.ax.T;
    t.ey = p.ay.T;
    t.ez = p.az.T;
    t.spec_off = 0;
    t.otf_off = 0;
    std::vector<int2> iz, ii;
    for (int p0 = 0; p0 < t.ty * t.px; p0 += kZChunk) iz.push_back(make_int2(0, p0));
    for (int z = 0; z < t.tz; ++z) ii.push_back(make_int2(0, z));
    a.lag_tile.alloc(sizeof(TileDesc));
    a.lag_items_z.alloc(iz.size() * sizeof(int2));
    a.lag_items_inv.alloc(ii.size() * sizeof(int2));
    upload_table(a.lag_tile.p, &t, sizeof(TileDesc));
    upload_table(a.lag_items_z.p, iz.data(), iz.size() * sizeof(int2));
    upload_table(a.lag_items_inv.p, ii.data(), ii.size() * sizeof(int2));
    a.n_lag_z = (int)iz.size();
    a.n_lag_inv = (int)ii.size();
    tile_max = std::max(tile_max, (long long)p.ax.T * p.ay.T * p.az.T);
    otf_max = std::max(otf_max, p.otf_elems);
  }
  long long spec_max = 0, kmax = 0;
  for (int v = 0; v < h->V; ++v) {
    spec_max = std::max(spec_max, h->plans[v]->spec_elems);
    kmax = std::max(kmax, vox(h->kd[v]));
  }
  h->r.alloc(h->N * sizeof(float));
  h->c_ext.alloc(ext_max * sizeof(float));
  h->spec_ext.alloc(spec_ext_max * sizeof(float2));
  h->spec_b.alloc(spec_max * sizeof(float2));
  h->acc.alloc(otf_max * sizeof(float2));
  h->lag_real.alloc(tile_max * sizeof(float));
  h->g_psi.alloc(h->N * sizeof(float));
  h->g_psf.alloc(kmax * sizeof(float));
  h->d_nll.alloc(sizeof(double));
  MVD_CHECK(cudaStreamSynchronize(h->stream));
}

// f_v = ext(psi) (*) kernel1_v; NLL epilogue (residual into h->r when `residual`)
void enqueue_blur_nll(mvd_decon* h, int v, bool residual) {
  const ConvPlan& p = *h->plans[v];
  float2* sp = h->spec.as<float2>();
  launch_fwd_mirror(h->pt, p, h->psi.as<float>(), sp, h->stream);
  launch_z(h->pt, p, sp, h->otf1[v].as<float2>(), h->stream);
  launch_inv_nll(h->pt, p, sp, h->img[v].as<float>(), h->w[v].as<float>(), residual ? h->r.as<float>() : nullptr,
                 h->d_nll.as<double>(), h->stream);
}

}  // namespace

extern "C" int mvd_forward(mvd_decon* h, double* nll) {
  MVD_API_BEGIN
  if (!h || !nll) return fail(MVD_ERR_ARG, "NULL argument");
  if (h->flags & MVD_FLAG_PLAIN) return fail(MVD_ERR_STATE, "forward/backward need the fused form");
  MVD_CHECK(cudaSetDevice(h->dev));
  adjoint_setup(h);
  MVD_CHECK(cudaMemsetAsync(h->d_nll.p, 0, sizeof(double), h->stream));
  for (int v = 0; v < h->V; ++v) enqueue_blur_nll(h, v, false);
  MVD_CHECK(cudaMemcpyAsync(nll, h->d_nll.p, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  MVD_CHECK(cudaStreamSynchronize(h->stream));
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_backward(mvd_decon* h, float* grad_psi, float* const* grad_psf) {
  MVD_API_BEGIN
  if (!h || !grad_psi || !grad_psf) return fail(MVD_ERR_ARG, "NULL argument");
  if (h->flags & MVD_FLAG_PLAIN) return fail(MVD_ERR_STATE, "forward/backward need the fused form");
  for (int v = 0; v < h->V; ++v)
    if (!grad_psf[v]) return fail(MVD_ERR_ARG, "NULL PSF gradient buffer");
  MVD_CHECK(cudaSetDevice(h->dev));
  adjoint_setup(h);
  cudaStream_t s = h->stream;
  MVD_CHECK(cudaMemsetAsync(h->g_psi.p, 0, h->N * sizeof(float), s));
  MVD_CHECK(cudaMemsetAsync(h->d_nll.p, 0, sizeof(double), s));
  MVD_CHECK(cudaMemsetAsync(h->r.p, 0, h->N * sizeof(float), s));  // zero outside the views' data boxes
  for (int v = 0; v < h->V; ++v) {
    const ConvPlan& p = *h->plans[v];
    mvd_decon::AdjView& a = h->adj[v];
    const auto& k = h->kd[v];
    // recompute this view's blur and residual (no blurred view is kept between calls)
    enqueue_blur_nll(h, v, true);
    // dNLL/dpsi: residual (zero outside) convolved with mirror(kernel1) on the extended grid,
    // then folded back through the mirror-single extension
    const ConvPlan& e = *a.ext;
    float2* se = h->spec_ext.as<float2>();
    launch_fwd_value_items(h->pt, e, e.d_tiles.as<TileDesc>(), e.d_items_fwd.as<int2>(), (int)e.items_fwd.size(),
                           h->r.as<float>(), h->dims[0], h->dims[1], h->dims[2], 0.f, se, s);
    launch_z(h->pt, e, se, a.otf_m.as<float2>(), s);
    const long long off = ((long long)(k[2] / 2) * e.ny + k[1] / 2) * e.nx + k[0] / 2;
    launch_inv_store_items(h->pt, e, e.d_tiles.as<TileDesc>(), e.d_items_inv.as<int2>(), (int)e.items_inv.size(),
                           se, h->c_ext.as<float>() + off, e.nx, e.ny, s);
    dev_fold_mirror(h->c_ext.as<float>(), e.nx, e.ny, a.fold_tab.as<int>(), h->dims[0], h->dims[1], h->dims[2],
                    h->g_psi.as<float>(), s);
    // dNLL/dP_v(j) = sum_x r(x) ext(psi)(x - (j - k/2)): per tile, spectrum of the residual
    // restricted to the effective region times the conjugate spectrum of ext(psi) over the
    // tile window, summed over tiles; one inverse transform; the kernel-sized lags
    float2* sa = h->spec.as<float2>();
    float2* sb = h->spec_b.as<float2>();
    launch_fwd_mirror(h->pt, p, h->psi.as<float>(), sa, s);
    launch_z_forward(h->pt, p, sa, s);
    launch_fwd_masked(h->pt, p, h->r.as<float>(), sb, s);
    launch_z_forward(h->pt, p, sb, s);
    dev_cross_accumulate(sb, sa, (int)p.tiles.size(), p.otf_elems, h->acc.as<float2>(), s);
    launch_z_inverse_items(h->pt, p, a.lag_tile.as<TileDesc>(), a.lag_items_z.as<int2>(), a.n_lag_z,
                           h->acc.as<float2>(), s);
    launch_inv_store_items(h->pt, p, a.lag_tile.as<TileDesc>(), a.lag_items_inv.as<int2>(), a.n_lag_inv,
                           h->acc.as<float2>(), h->lag_real.as<float>(), p.ax.T, p.ay.T, s);
    const double n_tile = (double)p.ax.T * p.ay.T * p.az.T;
    dev_extract_lags(h->lag_real.as<float>(), p.ax.T, p.ay.T, p.az.T, k[0], k[1], k[2], (float)(1.0 / n_tile),
                     h->g_psf.as<float>(), s);
    MVD_CHECK(cudaMemcpyAsync(grad_psf[v], h->g_psf.p, vox(k) * sizeof(float), cudaMemcpyDeviceToHost, s));
  }
  MVD_CHECK(cudaMemcpyAsync(grad_psi, h->g_psi.p, h->N * sizeof(float), cudaMemcpyDeviceToHost, s));
  MVD_CHECK(cudaStreamSynchronize(s));
  return MVD_OK;
  MVD_API_END
}

extern "C" int mvd_set_kernel(mvd_decon* h, int view, int which, const float* data) {
  MVD_API_BEGIN
  if (!h || !data) return fail(MVD_ERR_ARG, "NULL argument");
  if (view < 0 || view >= h->V || (which != 1 && which != 2)) return fail(MVD_ERR_ARG, "bad view or kernel");
  MVD_CHECK(cudaSetDevice(h->dev));
  AllocScope scope(h->stream);
  DevBuf& k = which == 1 ? h->k1[view] : h->k2[view];
  MVD_CHECK(cudaMemcpyAsync(k.p, data, vox(h->kd[view]) * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  const ConvPlan& p = *h->plans[view];
  build_otf(h->pt, p, k.as<float>(), (which == 1 ? h->otf1[view] : h->otf2[view]).as<float2>(), h->scratch,
            h->stream);
  if (which == 1 && !h->adj.empty()) {
    mvd_decon::AdjView& a = h->adj[view];
    DevBuf mk = mirrored(h, h->k1[view].as<float>(), h->kd[view]);
    build_otf(h->pt, *a.ext, mk.as<float>(), a.otf_m.as<float2>(), h->scratch, h->stream);
  }
  MVD_CHECK(cudaStreamSynchronize(h->stream));
  return MVD_OK;
  MVD_API_END
}
