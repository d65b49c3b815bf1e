// Host side of the tiled FFT convolution engine (internal C++ API; the C ABI is in capi.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "kernels.cuh"

namespace mvd {

struct CudaError : std::runtime_error {
  cudaError_t code;
  CudaError(cudaError_t c, const std::string& what) : std::runtime_error(what), code(c) {}
};

void check_cuda(cudaError_t e, const char* what);
#define MVD_CHECK(x) ::mvd::check_cuda((x), #x)

// 2,3,5-smooth helpers (the FFT radices are products of 2, 3 and 5)
bool is_smooth(int n);
int next_smooth(int n, bool even);
std::vector<int> factorize(int n);  // radices from {20,18,16,15,12,10,9,8,6,5,4,3,2}, product == n

// Device memory owned by RAII.  Allocated while an AllocScope is active on this thread, it
// comes from the device's memory pool in the scope stream's order (cudaMallocAsync) and is
// freed in that stream's order (cudaFreeAsync): no device-wide synchronisation, and the pool
// keeps the memory for the next allocation.  Otherwise plain cudaMalloc / cudaFree.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;  // the allocation's stream (stream-ordered), or none
  DevBuf() = default;
  explicit DevBuf(size_t b) { alloc(b); }
  ~DevBuf();
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes), stream(o.stream) {
    o.p = nullptr;
    o.bytes = 0;
    o.stream = nullptr;
  }
  DevBuf& operator=(DevBuf&& o) noexcept;
  void alloc(size_t b);
  void ensure(size_t b);  // grow (contents lost) if smaller
  void release();
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// Stream-ordered allocation for the DevBufs created on this thread during its lifetime; the
// stream must outlive them.  Host-to-device uploads of tables go through upload_table(), which is
// ordered in the same stream (a plain copy could overtake work still using recycled memory).
class AllocScope {
 public:
  explicit AllocScope(cudaStream_t s);
  ~AllocScope();
  AllocScope(const AllocScope&) = delete;
  AllocScope& operator=(const AllocScope&) = delete;
 private:
  cudaStream_t prev_;
};
cudaStream_t alloc_stream();
void upload_table(void* dst, const void* src, size_t bytes);
// Keep freed pool memory cached in this process instead of returning it at every
// synchronisation (the device's default pool; a process-local attribute).
void keep_pool_memory(int dev);

// Twiddle tables and FFT plans for every length used on a device.
class PlanTable {
 public:
  // creates the plan if needed (host side only); radices in the planner's descending order, or
  // ascending (a separate plan of the same length)
  int index_of(int n, bool ascending = false);
  const FftPlan* device();      // uploads if changed; valid until the next upload
  size_t size() const { return host_.size(); }
 private:
  static constexpr int kCapacity = 256;
  std::vector<FftPlan> host_;
  std::map<int, int> by_len_;
  std::vector<std::unique_ptr<DevBuf>> tw_bufs_;
  DevBuf dev_;
  bool dirty_ = true;
};

// One axis of a tile grid.
struct AxisTiles {
  int size = 0, k = 0, T = 0, n = 0, E = 0;
};

// A convolution plan over one volume with one kernel size: the tiles, their work items and
// the spectrum / OTF layout.
struct ConvPlan {
  int nx = 0, ny = 0, nz = 0;          // region the tiles cover (their effective regions)
  int kx = 0, ky = 0, kz = 0;          // kernel
  // the volume the gathers and epilogues address (tile coordinates are in its frame), and the
  // data box of a value-extended input (value outside it); by default the covered region
  int vol[3] = {0, 0, 0};
  int box_lo[3] = {0, 0, 0}, box_hi[3] = {0, 0, 0};
  AxisTiles ax, ay, az;
  std::vector<TileDesc> tiles;         // host copy
  std::vector<int2> items_fwd, items_inv, items_z;
  std::vector<int2> items_zw;          // z items of kZWideChunk pencils (the in-place z pass)
  long long spec_elems = 0;            // complex elements of all tile spectra
  long long otf_elems = 0;             // complex elements of one OTF (all tiles share the shape)
  size_t smem_plane = 0, smem_z = 0;
  int threads_plane = 0;               // CTA size of the plane kernels (a multiple of 32, <= kThreads)
  bool tensor_dft = false;             // z pass with its middle DFT stage on the tensor cores (if compiled)
  bool ascending = false;              // radices of every length in ascending order
  bool generic = false;                // run the generic kernels even where a compiled shape exists
  bool staged = false;                 // large compiled planes: in-place kernels, two CTAs per SM
  DevBuf d_tiles, d_items_fwd, d_items_inv, d_items_z, d_items_zw;
  // one tile of this shape at the origin and its work items: the OTF build's tables
  DevBuf d_otf_tile, d_otf_fwd, d_otf_z;
  int n_otf_fwd = 0, n_otf_z = 0;
  long long padded_voxels() const { return (long long)tiles.size() * ax.T * ay.T * az.T; }
  void upload();
};

struct PlanOptions {
  int force_tx = 0, force_ty = 0, force_tz = 0;  // 0 = planner's choice
  int cap = 0;                                   // plane-buffer budget; 0 = plane_cap()
  int threads = 0;                               // plane CTA size; 0 = plane_threads()
  bool ascending = false;                        // radix order of the tile's FFT lengths
  bool generic = false;                          // generic kernels only
};

// Move a plan's tiles by (dx, dy, dz) into the frame of a larger volume `vol` whose data box
// is the covered region (the tiles then cover [d, d + n) of that volume); re-uploads the tiles.
void place_plan(ConvPlan& p, int dx, int dy, int dz, const int vol[3]);

// Choose tiles for a (volume, kernel) pair; effective regions cover the whole volume.
std::unique_ptr<ConvPlan> make_conv_plan(PlanTable& pt, int nx, int ny, int nz, int kx, int ky,
                                         int kz, const PlanOptions& opt = PlanOptions());

// Planner's budget for one plane buffer (complex values).
int plane_cap();
// The default planner's limits: the largest plane buffer it considers (complex values), and
// the relative cost it gives a tile shape whose plane buffer holds `plane` complex values.
// Planes beyond two CTAs per SM (kPlaneCapDefault) cost 1.12 (one CTA per SM: the plane passes
// measured 16% slower at one 1024-thread CTA than at two 512-thread CTAs per SM), shapes without
// compile-time-shaped kernels 1.3 (the compiled ones measured 28-33% faster per launch); the
// large shapes with in-place kernels run two CTAs per SM and take no plane-size factor.  With
// MVD_PLANE_CAP set, that budget is a hard limit and every shape costs the same.
int plane_limit();
double plane_cost_factor(int tx, int ty, long long plane);
bool compiled_plane_shape(int tx, int ty);
// Default CTA size of the plane kernels (MVD_PLANE_THREADS overrides it).
int plane_threads();
// Whether compiled tile shapes use their compile-time-shaped plane kernels (MVD_FIXED_PLANES=0
// selects the generic kernels everywhere).
bool use_fixed_planes();
// Whether plans of the large compiled shapes run the in-place plane kernels (two CTAs per SM;
// MVD_STAGED_PLANES=0 selects the two-buffer kernels; the autotuner times both either way), and
// whether a shape has them.
bool use_staged_planes();
bool staged_plane_shape(int tx, int ty);
// L2 prefetch through tensor maps in the plane kernels (MVD_L2_PREFETCH=0 turns it off).
bool use_l2_prefetch();
// Whether pencils of length tz have a tensor-core z pass, and the number of its MMA waits that
// gave up on the current device since the last call (the counter is reset; zero when none ran).
bool tensor_dft_supported(int tz);
int tensor_dft_failures();
// Uploads the tensor-core z pass's DFT matrices for the current device (once; outside any stream
// capture, since it allocates).
void tensor_dft_prepare();
struct ConvPlan;
// Whether the plan's plane shape or pencil length has compiled kernels, and the CTA size of the
// compiled plane kernels of its shape (0 if none).
bool has_compiled_kernels(const ConvPlan& p);
// Whether the plan's plane shape has in-place (tensor-memory-staged) kernels for its rows.
bool has_staged_kernels(const ConvPlan& p);
int compiled_plane_threads(const ConvPlan& p);
// Tensor map of a float volume [nz][ny][nx] with a (w, h, 1) box (cached); false when the volume
// does not meet the tensor copy's rules (16-byte aligned base and row stride, box <= 256).
bool volume_box_map(const float* base, int nx, int ny, int nz, int w, int h, CUtensorMap* out);

// Describe the plan for logs.
std::string describe(const ConvPlan& p);

// Build the (scaled) spectrum of a kernel for the tile shape of `plan` into `otf`
// (plan.otf_elems complex values).  `kernel` is a device [kz][ky][kx] float array.  Enqueued
// on `s` without waiting; `scratch_real` must stay allocated until the work is done.
void build_otf(PlanTable& pt, const ConvPlan& plan, const float* kernel, float2* otf,
               DevBuf& scratch_real, cudaStream_t s);

enum class Ext { Mirror = 0, Value = 1 };

// Full convolution out = ext(in) (*) kernel over the volume (out may alias nothing in `in`).
void convolve(PlanTable& pt, const ConvPlan& plan, const float* in, Ext ext, float value,
              const float2* otf, float2* spec, float* out, cudaStream_t s);

// Raise a kernel's dynamic shared-memory limit (cached per device, kernel and size).
void set_smem_raw(const void* kernel, size_t bytes);
template <class K>
inline void set_smem(K kernel, size_t bytes) {
  set_smem_raw(reinterpret_cast<const void*>(kernel), bytes);
}

// Forward plane pass over explicit tile / item tables, gathering from a (vx, vy, vz) volume
// with a constant border value; and the forward-only, scaled z pass (OTF preparation).
void launch_fwd_value_items(PlanTable& pt, const ConvPlan& p, const TileDesc* tiles, const int2* items, int nitems,
                            const float* vol, int vx, int vy, int vz, float value, float2* spec, cudaStream_t s);
void launch_z_forward_scaled(PlanTable& pt, const ConvPlan& p, const TileDesc* tiles, const int2* items, int nitems,
                             float2* spec, float scale, cudaStream_t s);

// The three passes, for fused use by the deconvolution handle.
void launch_fwd_mirror(PlanTable& pt, const ConvPlan& p, const float* vol, float2* spec, cudaStream_t s);
void launch_fwd_value(PlanTable& pt, const ConvPlan& p, const float* vol, float value, float2* spec,
                      cudaStream_t s);
void launch_z(PlanTable& pt, const ConvPlan& p, float2* spec, const float2* otf, cudaStream_t s);
void launch_inv_store(PlanTable& pt, const ConvPlan& p, const float2* spec, float* out, cudaStream_t s);
void launch_inv_quotient(PlanTable& pt, const ConvPlan& p, const float2* spec, const float* img,
                         float* q, cudaStream_t s);
void launch_inv_update(PlanTable& pt, const ConvPlan& p, const float2* spec, float* psi,
                       const float* weight, float lambda, double* stat_sum, unsigned* stat_max,
                       const StatArchive& archive, cudaStream_t s);

// Kernel launches issued by this library (all devices), for launch accounting.
long long launch_count();
void count_launch(int n = 1);

// ---- forward/backward of the Poisson image-formation model (adjoint.cu, passes_*.cu) ----
// forward plane pass of `vol` (value 0 outside) keeping only each tile's effective region
void launch_fwd_masked(PlanTable& pt, const ConvPlan& p, const float* vol, float2* spec, cudaStream_t s);
// forward-only z pass (unscaled) over every tile of p
void launch_z_forward(PlanTable& pt, const ConvPlan& p, float2* spec, cudaStream_t s);
// inverse-only z pass over explicit tables
void launch_z_inverse_items(PlanTable& pt, const ConvPlan& p, const TileDesc* tiles, const int2* items, int nitems,
                            float2* spec, cudaStream_t s);
// inverse plane pass storing the effective region of explicit tiles into out (dims nx, ny)
void launch_inv_store_items(PlanTable& pt, const ConvPlan& p, const TileDesc* tiles, const int2* items, int nitems,
                            const float2* spec, float* out, int nx, int ny, cudaStream_t s);
// inverse plane pass with the NLL epilogue: nll += sum, r = residual (r may be null)
void launch_inv_nll(PlanTable& pt, const ConvPlan& p, const float2* spec, const float* img, const float* w, float* r,
                    double* nll, cudaStream_t s);
// acc[i] = sum_t B_t[i] conj(A_t[i]) over `ntiles` tile spectra of `elems` values each
void dev_cross_accumulate(const float2* B, const float2* A, int ntiles, long long elems, float2* acc, cudaStream_t s);
// G[j] = scale * R[(j - k/2) mod T] for the kernel-sized output G (circular lags of a tile)
void dev_extract_lags(const float* R, int tx, int ty, int tz, int kx, int ky, int kz, float scale, float* G,
                      cudaStream_t s);
// g[y] += sum of c over the extended positions that mirror-single maps to y; the tables list,
// per axis, for each y in [0, n) the extended indices (CSR: start[n + 1], idx[]).
void dev_fold_mirror(const float* c, int nxe, int nye, const int* tab, int nx, int ny, int nz, float* g,
                     cudaStream_t s);
// host: CSR tables of the mirror fold for an axis of n voxels extended by h on both sides
void mirror_fold_table(int n, int h, std::vector<int>& start, std::vector<int>& idx);

// bounding box of the voxels with img > 0 or w > 0: box[0..2] = min (x, y, z), box[3..5] = max
// (atomics into `box`, which must hold {INT_MAX x3, -1 x3} before the call)
void dev_data_box(const float* img, const float* w, int nx, int ny, int nz, int* box, cudaStream_t s);

// ---- elementwise / reduction helpers (misc kernels) ----
void dev_sum_f64(const float* x, long long n, double* out_dev, cudaStream_t s);  // *out += sum
void dev_scale_div(float* x, long long n, const double* div_dev, cudaStream_t s); // x = (float)(x / d)
void dev_mirror(const float* in, float* out, int nx, int ny, int nz, cudaStream_t s);
void dev_mul(float* a, const float* b, long long n, cudaStream_t s);
void dev_pow(float* a, int power, long long n, cudaStream_t s);
void dev_fill(float* a, float v, long long n, cudaStream_t s);
void dev_first_iteration(const float* const* views, int nviews, long long n, double* sum_count,
                         cudaStream_t s);  // sum_count[0] += sum of means, [1] += count
void dev_fill_from_avg(float* psi, const double* sum_count, long long n, cudaStream_t s);
void dev_mask(float* psi, const float* const* views, int nviews, long long n, cudaStream_t s);
void dev_quotient(float* blurred_to_q, const float* img, long long n, cudaStream_t s);
void dev_update(float* psi, const float* integral, const float* weight, float lambda, long long n,
                double* stat_sum, unsigned* stat_max, cudaStream_t s);
// block copy / paste of the reference's Block.copyBlock / pasteBlock
void dev_copy_block(const float* vol, int nx, int ny, int nz, float* block, int bx, int by, int bz,
                    int ox, int oy, int oz, Ext ext, float value, cudaStream_t s);
void dev_paste_block(const float* block, int bx, int by, int bz, int lx, int ly, int lz, float* vol,
                     int nx, int ny, int nz, int ex0, int ey0, int ez0, int sx, int sy, int sz,
                     cudaStream_t s);

}  // namespace mvd
