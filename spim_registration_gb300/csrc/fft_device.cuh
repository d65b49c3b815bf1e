// Block-cooperative mixed-radix Stockham FFT in shared memory (FP32), sm_103a.
//
// One CTA transforms `count` independent complex sequences of length N that live in shared
// memory at  d[batch * bs + n * es].  Each stage of radix R reads a butterfly's R inputs into
// registers, twiddles, runs the R-point DFT in registers and writes the R outputs to the
// other of two buffers in Stockham (self-sorting) order, so no bit-reversal pass is needed
// and a thread never holds more than one butterfly.  Butterflies are assigned batch-fastest,
// which makes both row transforms (es = 1, odd bs) and column transforms (bs = 1) free of
// shared-memory bank conflicts.
//
// Radices: 2, 3, 4, 5, 7, 8.  Twiddles come from a per-length table exp(-2 pi i k / N) that
// the host computes in double precision.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mvd {

constexpr int kMaxStages = 12;

// Runtime plan of one transform length (device copy lives in a plan table).
struct FftPlan {
  int n;                    // transform length
  int nstages;              // number of radix stages
  int radix[kMaxStages];    // radices, product == n
  const float2* tw;         // exp(-2 pi i k / n), k in [0, n)
  const float2* tw_r2c;     // for the real-input length 2n: exp(-2 pi i k / (2n)), k in [0, n]
};

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---------------------------------------------------------------------------------------
// R-point DFTs in registers.  Forward uses exp(-2 pi i / R); inverse the conjugate root.
// ---------------------------------------------------------------------------------------
template <int R, bool INV>
struct Dft;

template <bool INV>
struct Dft<2, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool INV>
struct Dft<4, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    float2 s0 = cadd(v[0], v[2]), d0 = csub(v[0], v[2]);
    float2 s1 = cadd(v[1], v[3]), d1 = mul_mi<INV>(csub(v[1], v[3]));
    v[0] = cadd(s0, s1);
    v[2] = csub(s0, s1);
    v[1] = cadd(d0, d1);
    v[3] = csub(d0, d1);
  }
};

template <bool INV>
struct Dft<8, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    const float h = 0.70710678118654752440f;  // sqrt(1/2)
    // radix-2 split: even / odd samples, then two 4-point DFTs
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    // twiddles w8^k for k = 1..3 (forward: exp(-i pi k / 4))
    float2 o1 = o[1], o2 = o[2], o3 = o[3];
    o[1] = INV ? make_float2(h * (o1.x - o1.y), h * (o1.x + o1.y))
               : make_float2(h * (o1.x + o1.y), h * (o1.y - o1.x));
    o[2] = mul_mi<INV>(o2);
    o[3] = INV ? make_float2(-h * (o3.x + o3.y), h * (o3.x - o3.y))
               : make_float2(h * (o3.y - o3.x), -h * (o3.x + o3.y));
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = cadd(e[k], o[k]);
      v[k + 4] = csub(e[k], o[k]);
    }
  }
};

template <bool INV>
struct Dft<3, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    const float c = -0.5f;
    const float s = 0.86602540378443864676f;  // sin(2 pi / 3)
    float2 a = cadd(v[1], v[2]);
    float2 b = csub(v[1], v[2]);
    float2 t = make_float2(v[0].x + c * a.x, v[0].y + c * a.y);
    float2 u = mul_mi<INV>(cscale(b, s));
    v[0] = cadd(v[0], a);
    v[1] = cadd(t, u);
    v[2] = csub(t, u);
  }
};

template <bool INV>
struct Dft<5, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    const float c1 = 0.30901699437494742410f;   // cos(2 pi / 5)
    const float c2 = -0.80901699437494742410f;  // cos(4 pi / 5)
    const float s1 = 0.95105651629515357212f;   // sin(2 pi / 5)
    const float s2 = 0.58778525229247312917f;   // sin(4 pi / 5)
    float2 p1 = cadd(v[1], v[4]), m1 = csub(v[1], v[4]);
    float2 p2 = cadd(v[2], v[3]), m2 = csub(v[2], v[3]);
    float2 x0 = v[0];
    float2 a1 = make_float2(x0.x + c1 * p1.x + c2 * p2.x, x0.y + c1 * p1.y + c2 * p2.y);
    float2 a2 = make_float2(x0.x + c2 * p1.x + c1 * p2.x, x0.y + c2 * p1.y + c1 * p2.y);
    float2 b1 = make_float2(s1 * m1.x + s2 * m2.x, s1 * m1.y + s2 * m2.y);
    float2 b2 = make_float2(s2 * m1.x - s1 * m2.x, s2 * m1.y - s1 * m2.y);
    float2 jb1 = mul_mi<INV>(b1), jb2 = mul_mi<INV>(b2);
    v[0] = make_float2(x0.x + p1.x + p2.x, x0.y + p1.y + p2.y);
    v[1] = cadd(a1, jb1);
    v[4] = csub(a1, jb1);
    v[2] = cadd(a2, jb2);
    v[3] = csub(a2, jb2);
  }
};

template <bool INV>
struct Dft<7, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    // cos / sin of 2 pi k / 7, k = 1..3
    const float c[3] = {0.62348980185873353053f, -0.22252093395631440429f, -0.90096886790241912624f};
    const float s[3] = {0.78183148246802980871f, 0.97492791218182360702f, 0.43388373911755812048f};
    float2 p[3], m[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      p[k] = cadd(v[k + 1], v[6 - k]);
      m[k] = csub(v[k + 1], v[6 - k]);
    }
    float2 x0 = v[0];
    float2 out[7];
    out[0] = make_float2(x0.x + p[0].x + p[1].x + p[2].x, x0.y + p[0].y + p[1].y + p[2].y);
#pragma unroll
    for (int k = 1; k <= 3; ++k) {
      float2 a = x0, b = make_float2(0.f, 0.f);
#pragma unroll
      for (int n = 1; n <= 3; ++n) {
        const int idx = (k * n) % 7;  // cos(2 pi k n / 7) = c[min(idx, 7-idx) - 1]
        const int j = (idx <= 3 ? idx : 7 - idx) - 1;
        const float sg = idx <= 3 ? 1.f : -1.f;  // sin(2 pi k n / 7) sign
        a.x += c[j] * p[n - 1].x;
        a.y += c[j] * p[n - 1].y;
        b.x += sg * s[j] * m[n - 1].x;
        b.y += sg * s[j] * m[n - 1].y;
      }
      float2 jb = mul_mi<INV>(b);
      out[k] = cadd(a, jb);
      out[7 - k] = csub(a, jb);
    }
#pragma unroll
    for (int k = 0; k < 7; ++k) v[k] = out[k];
  }
};

// ---------------------------------------------------------------------------------------
// One Stockham stage of radix R, out of place (src -> dst), no barrier inside.
// Butterfly b of `count` sequences: batch = b % count (fastest), j = b / count.
// ---------------------------------------------------------------------------------------
template <int R, bool INV>
__device__ __forceinline__ void stockham_stage(const float2* __restrict__ src, float2* __restrict__ dst, int N,
                                               int Ns, int count, int es, int bs,
                                               const float2* __restrict__ tw) {
  const int NR = N / R;
  const int nb = count * NR;
  const int twstride = N / (Ns * R);
#pragma unroll 2
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const int j = b / count;
    const int batch = b - j * count;
    const float2* s = src + batch * bs + j * es;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[r * NR * es];
    const int k = j % Ns;
    if (k != 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 w = __ldg(tw + r * k * twstride);
        if (INV) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    Dft<R, INV>::run(v);
    float2* d = dst + batch * bs + ((j - k) * R + k) * es;
#pragma unroll
    for (int r = 0; r < R; ++r) d[r * Ns * es] = v[r];
  }
}

// Full transform of `count` sequences with the plan `p` (read from global memory), ping-pong
// between the buffers `cur` and `oth`; on return `cur` holds the result.
template <bool INV>
__device__ __forceinline__ void block_fft(float2*& cur, float2*& oth, const FftPlan* __restrict__ p, int count,
                                          int es, int bs) {
  const int n = __ldg(&p->n);
  const int ns = __ldg(&p->nstages);
  const float2* tw = p->tw;
  int Ns = 1;
  for (int s = 0; s < ns; ++s) {
    const int R = __ldg(&p->radix[s]);
    switch (R) {
      case 2: stockham_stage<2, INV>(cur, oth, n, Ns, count, es, bs, tw); break;
      case 3: stockham_stage<3, INV>(cur, oth, n, Ns, count, es, bs, tw); break;
      case 4: stockham_stage<4, INV>(cur, oth, n, Ns, count, es, bs, tw); break;
      case 5: stockham_stage<5, INV>(cur, oth, n, Ns, count, es, bs, tw); break;
      case 7: stockham_stage<7, INV>(cur, oth, n, Ns, count, es, bs, tw); break;
      default: stockham_stage<8, INV>(cur, oth, n, Ns, count, es, bs, tw); break;
    }
    __syncthreads();
    float2* t = cur;
    cur = oth;
    oth = t;
    Ns *= R;
  }
}

// ---------------------------------------------------------------------------------------
// Real <-> half-complex post/pre-processing of rows.  A row of 2M reals packed as M complex
// values z[n] = x[2n] + i x[2n+1] was transformed to Z = FFT_M(z); the post-step turns it
// into X[k], k = 0..M, of the length-2M real transform, writing X[M] to slot M.
// The pre-step is its inverse up to a factor 2 (together with an unnormalised inverse
// FFT_M it yields 2M * x).  `tw2` = exp(-2 pi i k / (2M)), k in [0, M].
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void r2c_post(float2* d, int rows, int M, int pitch,
                                         const float2* __restrict__ tw2) {
  const int half = M / 2;  // pairs (k, M-k) for k = 0..half
  const int total = rows * (half + 1);
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int row = i % rows;
    const int k = i / rows;
    float2* r = d + row * pitch;
    if (k == 0) {
      float2 z0 = r[0];
      r[0] = make_float2(z0.x + z0.y, 0.f);
      r[M] = make_float2(z0.x - z0.y, 0.f);
      continue;
    }
    const int k2 = M - k;
    float2 zk = r[k], zc = r[k2];
    // X[k] = (Zk + conj(Zc))/2 - i/2 * w^k (Zk - conj(Zc))
    float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y - zc.y));
    float2 o = make_float2(0.5f * (zk.x - zc.x), 0.5f * (zk.y + zc.y));  // (Zk - conj Zc)/2
    float2 w = __ldg(tw2 + k);
    float2 wo = cmul(w, o);
    float2 xk = make_float2(e.x + wo.y, e.y - wo.x);  // e - i * wo
    if (k2 == k) {
      r[k] = xk;
    } else {
      // X[M-k] = conj(e) - i conj(w^k o)   (uses w^{M-k} = -conj(w^k))
      float2 xk2 = make_float2(e.x - wo.y, -e.y - wo.x);
      r[k] = xk;
      r[k2] = xk2;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ void c2r_pre(float2* d, int rows, int M, int pitch,
                                        const float2* __restrict__ tw2) {
  const int half = M / 2;
  const int total = rows * (half + 1);
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int row = i % rows;
    const int k = i / rows;
    float2* r = d + row * pitch;
    if (k == 0) {
      float2 x0 = r[0], xm = r[M];
      // Z[0] = (X0 + conj XM) + i (X0 - conj XM)
      float2 e = make_float2(x0.x + xm.x, x0.y - xm.y);
      float2 o = make_float2(x0.x - xm.x, x0.y + xm.y);
      r[0] = make_float2(e.x - o.y, e.y + o.x);
      continue;
    }
    const int k2 = M - k;
    float2 xk = r[k], xc = r[k2];
    // Z[k] = (Xk + conj Xc) + i conj(w^k) (Xk - conj Xc)
    float2 e = make_float2(xk.x + xc.x, xk.y - xc.y);
    float2 o = make_float2(xk.x - xc.x, xk.y + xc.y);
    float2 w = __ldg(tw2 + k);
    float2 wo = cmul(cconj(w), o);
    float2 zk = make_float2(e.x - wo.y, e.y + wo.x);
    if (k2 == k) {
      r[k] = zk;
    } else {
      // Z[M-k] = conj(e) + i w^k conj(o)   (uses conj(w^{M-k}) = -w^k)
      float2 wo2 = cmul(w, cconj(o));
      float2 zk2 = make_float2(e.x - wo2.y, -e.y + wo2.x);
      r[k] = zk;
      r[k2] = zk2;
    }
  }
  __syncthreads();
}

}  // namespace mvd
