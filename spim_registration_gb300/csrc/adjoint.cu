// Small kernels of the forward/backward pair of the Poisson image-formation model:
// cross-spectrum accumulation and lag extraction (PSF gradient), mirror fold (psi gradient).
#include "engine.h"

namespace mvd {

static int grid1(long long n) {
  long long b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152LL * 16 ? 152LL * 16 : b));
}

__global__ void cross_accumulate_kernel(const float2* __restrict__ B, const float2* __restrict__ A, int ntiles,
                                        long long elems, float2* __restrict__ acc) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < elems; i += (long long)gridDim.x * blockDim.x) {
    float2 s = make_float2(0.f, 0.f);
    for (int t = 0; t < ntiles; ++t) {
      const float2 b = __ldg(B + t * elems + i), a = __ldg(A + t * elems + i);
      // b * conj(a)
      s.x += b.x * a.x + b.y * a.y;
      s.y += b.y * a.x - b.x * a.y;
    }
    acc[i] = s;
  }
}

void dev_cross_accumulate(const float2* B, const float2* A, int ntiles, long long elems, float2* acc, cudaStream_t s) {
  cross_accumulate_kernel<<<grid1(elems), 256, 0, s>>>(B, A, ntiles, elems, acc);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

__global__ void extract_lags_kernel(const float* __restrict__ R, int tx, int ty, int tz, int kx, int ky, int kz,
                                    float scale, float* __restrict__ G) {
  const long long n = (long long)kx * ky * kz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int jx = (int)(i % kx), jy = (int)((i / kx) % ky), jz = (int)(i / ((long long)kx * ky));
    const int lx = ((jx - kx / 2) % tx + tx) % tx;
    const int ly = ((jy - ky / 2) % ty + ty) % ty;
    const int lz = ((jz - kz / 2) % tz + tz) % tz;
    G[i] = scale * R[((long long)lz * ty + ly) * tx + lx];
  }
}

void dev_extract_lags(const float* R, int tx, int ty, int tz, int kx, int ky, int kz, float scale, float* G,
                      cudaStream_t s) {
  extract_lags_kernel<<<grid1((long long)kx * ky * kz), 256, 0, s>>>(R, tx, ty, tz, kx, ky, kz, scale, G);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

// tab layout: [sx (nx+1) | ix | sy (ny+1) | iy | sz (nz+1) | iz] with the idx lengths nx+2hx etc.
__global__ void fold_mirror_kernel(const float* __restrict__ c, int nxe, int nye, const int* __restrict__ sx,
                                   const int* __restrict__ ix, const int* __restrict__ sy, const int* __restrict__ iy,
                                   const int* __restrict__ sz, const int* __restrict__ iz, int nx, int ny, int nz,
                                   float* __restrict__ g) {
  const long long n = (long long)nx * ny * nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long long)nx * ny));
    float acc = 0.f;
    for (int a = sz[z]; a < sz[z + 1]; ++a)
      for (int b = sy[y]; b < sy[y + 1]; ++b) {
        const float* row = c + ((long long)iz[a] * nye + iy[b]) * nxe;
        for (int e = sx[x]; e < sx[x + 1]; ++e) acc += row[ix[e]];
      }
    g[i] += acc;
  }
}

void dev_fold_mirror(const float* c, int nxe, int nye, const int* tab, int nx, int ny, int nz, float* g,
                     cudaStream_t s) {
  const int nze_unused = 0;
  (void)nze_unused;
  const int* sx = tab;
  const int* ix = sx + nx + 1;
  const int* sy = ix + nxe;
  const int* iy = sy + ny + 1;
  const int* sz = iy + nye;
  const int* iz = sz + nz + 1;
  fold_mirror_kernel<<<grid1((long long)nx * ny * nz), 256, 0, s>>>(c, nxe, nye, sx, ix, sy, iy, sz, iz, nx, ny, nz, g);
  MVD_CHECK(cudaGetLastError());
  count_launch();
}

void mirror_fold_table(int n, int h, std::vector<int>& start, std::vector<int>& idx) {
  std::vector<std::vector<int>> lists(n);
  for (int u = -h; u < n + h; ++u) {
    int y;
    if (n == 1) {
      y = 0;
    } else {
      const int period = 2 * n - 2;
      int m = u % period;
      if (m < 0) m += period;
      y = m < n ? m : period - m;
    }
    lists[y].push_back(u + h);
  }
  start.assign(n + 1, 0);
  idx.clear();
  for (int y = 0; y < n; ++y) {
    start[y] = (int)idx.size();
    idx.insert(idx.end(), lists[y].begin(), lists[y].end());
  }
  start[n] = (int)idx.size();
}

}  // namespace mvd
